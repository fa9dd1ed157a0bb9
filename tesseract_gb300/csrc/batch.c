/* The batched engine's host side: packs many enumeration jobs (verify, equiv, search) into one
   set of device arrays, cuts them into work units, runs the persistent interpreter kernel
   (batch_kernels.cu) and turns its counters back into one EnumResult per job, with the same
   fields, hits, 16 smallest hits and ops accounting as enum_run (src/enum.c:244-332).

   Nothing here is compiled per program, so thousands of different programs cost a few persistent
   launches.  Jobs routed to the interpreter whose cells do not fit its slot space (255 slots per
   job), or that ask for --part shares, are refused with an error; cuda_enum_run handles those. */
#include <stdlib.h>
#include <unistd.h>
#include <string.h>

#include <math.h>
#include <pthread.h>

#include "batch.h"
#include "engine.h"
#include "lutmap.h"


int tc_batch_launch(const struct TcBatchDev *d, int slots, cudaStream_t stream, double share,
                    int *grid_out, char *err, size_t errlen);

typedef struct TcWave TcWave;
void tc_wave_free(TcWave *w);

typedef struct {
    void  *p;
    size_t n, cap, elem;
} Vec;

static size_t vpush(Vec *v, const void *x, size_t count)
{
    if (v->n + count > v->cap) {
        v->cap = v->cap ? 2 * v->cap : 1024;
        while (v->cap < v->n + count)
            v->cap *= 2;
        v->p = tc_xrealloc(v->p, v->cap * v->elem);
    }
    memcpy((char *)v->p + v->n * v->elem, x, count * v->elem);
    size_t at = v->n;
    v->n += count;
    return at;
}

/* Packs program p (its cell c in slot base + c) into bundles: each run of NANDs then STOs,
   up to 4 and 3 per bundle. */
static uint32_t pack_code(Vec *code, const Program *p, unsigned base, uint32_t *count)
{
    uint32_t first = (uint32_t)code->n, nb = 0;
    size_t i = 0;
    while (i < p->len) {
        uint32_t nN = 0, nS = 0;
        uint8_t a[4] = {0, 0, 0, 0}, s[3] = {0, 0, 0};
        while (i < p->len && p->code[i].op == OP_NAND && nN < 4)
            a[nN++] = (uint8_t)(base + p->code[i++].addr);
        while (i < p->len && p->code[i].op == OP_STO && nS < 3) {
            if (!tc_program_readonly(p, p->code[i].addr))
                s[nS++] = (uint8_t)(base + p->code[i].addr);
            i++;
            if (i < p->len && p->code[i].op == OP_NAND)
                break;
        }
        uint64_t b = (uint64_t)(nN | nS << 4) | (uint64_t)a[0] << 8 | (uint64_t)a[1] << 16 |
                     (uint64_t)a[2] << 24 | (uint64_t)a[3] << 32 | (uint64_t)s[0] << 40 |
                     (uint64_t)s[1] << 48 | (uint64_t)s[2] << 56;
        vpush(code, &b, 1);
        nb++;
    }
    *count = nb;
    return first;
}

/* Cells that must be 0 before each assignment: read before written, or compared and never
   written (src/enum.c:90-111 resets the first kind; the second keep their power-on 0). */
static void clear_list(Vec *lists, const Program *p, unsigned base, const unsigned char *is_input,
                       uint16_t *n)
{
    unsigned char *seen = tc_xcalloc(p->ncells + 1, 1);
    for (size_t i = 0; i < p->len; i++) {
        uint32_t c = p->code[i].addr;
        if (c < CELL_FIRST_FREE || seen[c] || is_input[c])
            continue;
        seen[c] = p->code[i].op == OP_NAND ? 2 : 1;
    }
    for (uint32_t c = CELL_FIRST_FREE; c < p->ncells; c++)
        if (!is_input[c] && seen[c] != 1) {  /* read first, or never touched */
            uint16_t s = (uint16_t)(base + c);
            vpush(lists, &s, 1);
            (*n)++;
        }
    free(seen);
}

#define MAX_CLASSES 16

typedef struct {
    Vec jobs, code, luts, lists, rpn, vars;
    uint32_t units, unit_words;
    int      slots;
    /* units in launch order: class by class (jobs needing few shared-memory slots first), each
       class one launch with its own slot count, so light jobs run with more blocks per SM */
    int      nclass;
    uint32_t class_end[MAX_CLASSES];  /* units of classes 0..i end at class_end[i] */
    int      class_slots[MAX_CLASSES];
} Pack;

/* ---- LUT jobs: one tick, the pass mapped onto 3-input LUTs ------------------------------------ */

typedef struct {
    uint32_t *ops;        /* four words per LUT */
    int       nops, slots, ok;
    uint16_t *in_slot;    /* slot of input k */
    uint16_t *cmp;        /* the compare list, in the bundle format's layout */
    int       ncmp;       /* entries */
} LutJob;

static int net_or(TcNet *t, int a, int b)
{
    return tc_net_nand(t, tc_net_not(t, a), tc_net_not(t, b));
}

static int net_xor(TcNet *t, int a, int b)
{
    int n = tc_net_nand(t, a, b);
    return tc_net_nand(t, tc_net_nand(t, a, n), tc_net_nand(t, b, n));
}

typedef struct {
    int    node;
    double key;
} Keyed;

static int by_key(const void *x, const void *y)
{
    const Keyed *a = x, *b = y;
    return a->key < b->key ? -1 : a->key > b->key ? 1 : a->node - b->node;
}

/* Maps job e onto LUTs and gives every value a slot (linear scan: a slot is free again after
   the last op that reads it).  lj->ok = 0 when it does not fit 255 slots.

   Equiv and search fold their compare into the network: an accumulator ORs in each output's
   mismatch (a ^ b for a pair, v ^ target bit for search) as soon as the output's final value
   exists, so outputs do not stay live to the end of the pass (random programs output every
   cell), and the LUTs run in program order with each accumulator step placed right after the
   later of its operands.  The kernel then reads one mismatch word. */
static void lut_job(const Enum *e, const int *in_map, const int *out_map, LutJob *lj)
{
    const Program *a = e->a, *b = e->b;
    size_t n = a->ninputs;
    memset(lj, 0, sizeof *lj);
    TcNet *net = tc_net_new();
    int *leaf = tc_xmalloc((n + 1) * sizeof *leaf);
    for (size_t k = 0; k < n; k++)
        leaf[k] = tc_net_leaf(net, (int)k);
    int *cur_a = tc_xmalloc((a->ncells + 1) * sizeof *cur_a), *cur_b = NULL;
    tc_net_pass(net, a, a->inputs, n, leaf, cur_a);
    int a_end = tc_net_size(net), b_end = a_end;
    const TcSpec *sp = (const TcSpec *)e->spec;
    int *want = tc_xmalloc(((size_t)a->noutputs * 2 + 66) * sizeof *want), nwant = 0;
    if (e->mode == EN_EQUIV) {
        uint32_t *b_in = tc_xmalloc((n + 1) * sizeof *b_in);
        for (size_t k = 0; k < n; k++)
            b_in[k] = b->inputs[in_map[k]];
        cur_b = tc_xmalloc((b->ncells + 1) * sizeof *cur_b);
        tc_net_pass(net, b, b_in, n, leaf, cur_b);
        b_end = tc_net_size(net);
        free(b_in);
        for (size_t o = 0; o < a->noutputs; o++) {
            want[nwant++] = cur_a[a->outputs[o]];
            want[nwant++] = cur_b[b->outputs[out_map[o]]];
        }
    } else {
        for (int i = 0; i < sp->width; i++)
            want[nwant++] = cur_a[sp->out[i]];
    }
    if (e->mode != EN_VERIFY) {
        /* outputs in the order their values were made; the accumulator follows them */
        Keyed *ko = tc_xmalloc(((size_t)nwant + 1) * sizeof *ko);
        int nk = 0;
        if (e->mode == EN_EQUIV) {
            for (int i = 0; i < nwant; i += 2) {
                ko[nk].node = i;
                ko[nk++].key = want[i] > want[i + 1] ? want[i] : want[i + 1];
            }
        } else {
            for (int i = 0; i < nwant; i++) {
                ko[nk].node = i;
                ko[nk++].key = want[i];
            }
        }
        qsort(ko, (size_t)nk, sizeof *ko, by_key);
        uint64_t target = e->mode == EN_SEARCH ? cuda_spec_value(e->spec, 0) : 0;
        int acc = 0;
        for (int k = 0; k < nk; k++) {
            int i = ko[k].node;
            if (e->mode == EN_EQUIV && want[i] == want[i + 1])
                continue;  /* the same node: equal by construction */
            int d = e->mode == EN_EQUIV ? net_xor(net, want[i], want[i + 1])
                    : ((target >> i) & 1) ? tc_net_not(net, want[i]) : want[i];
            acc = net_or(net, acc, d);
        }
        free(ko);
        want[0] = acc;
        nwant = 1;
    }
    int size = tc_net_size(net);
    int *order = tc_xmalloc(((size_t)size + 1) * sizeof *order), norder = 0;
    tc_net_map(net, want, nwant, order, &norder);
    {
        /* the two programs side by side, each LUT at its place in its own program (the
           fraction of that program's network before it), and never before its operands, so an
           accumulator LUT comes right after the later of its operands */
        double *key = tc_xcalloc((size_t)size + 1, sizeof *key);
        Keyed *ko = tc_xmalloc(((size_t)norder + 1) * sizeof *ko);
        int lv[3], nlv;
        uint8_t t8;
        for (int q = 0; q < norder; q++) {
            int v = order[q];
            double k = v < a_end ? (double)v / a_end
                     : v < b_end ? (double)(v - a_end) / (b_end - a_end) : 0.0;
            tc_net_lut(net, v, lv, &nlv, &t8);
            for (int j = 0; j < nlv; j++)
                if (key[lv[j]] + 1e-9 > k)
                    k = key[lv[j]] + 1e-9;
            key[v] = k;
            ko[q].node = v;
            ko[q].key = k;
        }
        qsort(ko, (size_t)norder, sizeof *ko, by_key);
        for (int q = 0; q < norder; q++)
            order[q] = ko[q].node;
        free(ko);
        free(key);
    }
    /* last use of every value: the position of the last op reading it; outputs live to the end */
    int *last = tc_xmalloc(((size_t)size + 1) * sizeof *last);
    for (int i = 0; i < size; i++)
        last[i] = -1;
    int leaves[3], nl;
    uint8_t tt;
    for (int p = 0; p < norder; p++) {
        tc_net_lut(net, order[p], leaves, &nl, &tt);
        for (int j = 0; j < nl; j++)
            last[leaves[j]] = p;
    }
    for (int i = 0; i < nwant; i++)
        last[want[i]] = norder;
    int *slot = tc_xmalloc(((size_t)size + 1) * sizeof *slot);
    for (int i = 0; i < size; i++)
        slot[i] = -1;
    slot[0] = 0;
    slot[1] = 1;
    for (size_t k = 0; k < n; k++)
        slot[leaf[k]] = 2 + (int)k;
    int next = 2 + (int)n, nfree = 0;
    int *freed = tc_xmalloc(((size_t)norder + n + 1) * sizeof *freed);  /* values and inputs */
    lj->ops = tc_xmalloc(((size_t)norder + 1) * 4 * sizeof *lj->ops);
    lj->ok = next <= TC_BATCH_MAX_SLOTS;
    for (int p = 0; p < norder && lj->ok; p++) {
        tc_net_lut(net, order[p], leaves, &nl, &tt);
        int opslot[3];
        for (int j = 0; j < 3; j++)
            opslot[j] = j < nl ? slot[leaves[j]] : 0;
        for (int j = 0; j < nl; j++) {  /* operands read for the last time free their slots */
            int v = leaves[j];
            const TcNode *x = tc_net_node(net, v);
            int dup = 0;
            for (int q = 0; q < j; q++)
                dup |= leaves[q] == v;
            if (!dup && last[v] == p && x->kind != TN_CONST)
                freed[nfree++] = slot[v];  /* inputs too: they are rewritten every word */
        }
        int d = nfree ? freed[--nfree] : next++;
        if (d > TC_BATCH_MAX_SLOTS - 1) {
            lj->ok = 0;
            break;
        }
        slot[order[p]] = d;
        uint32_t *o = lj->ops + 4 * (size_t)p;
        o[0] = (uint32_t)opslot[0] * TC_BATCH_BLOCK * 4;
        o[1] = (uint32_t)opslot[1] * TC_BATCH_BLOCK * 4;
        o[2] = (uint32_t)opslot[2] * TC_BATCH_BLOCK * 4;
        o[3] = (uint32_t)d * TC_BATCH_BLOCK * 4 | (uint32_t)tt << 24;
    }
    lj->nops = norder;
    lj->slots = next;
    if (lj->ok) {
        lj->in_slot = tc_xmalloc((n + 1) * sizeof *lj->in_slot);
        for (size_t k = 0; k < n; k++)
            lj->in_slot[k] = (uint16_t)(2 + k);
        lj->cmp = tc_xmalloc(((size_t)nwant * 2 + 2) * sizeof *lj->cmp);
        if (e->mode == EN_EQUIV) {
            /* one pair: the mismatch accumulator against the constant-0 slot */
            lj->cmp[lj->ncmp++] = (uint16_t)slot[want[0]];
            lj->cmp[lj->ncmp++] = 0;
        } else if (e->mode == EN_SEARCH) {
            /* hits where the accumulator is 0: its complement, as target bit 0 */
            lj->cmp[lj->ncmp++] = (uint16_t)slot[want[0]];
            lj->cmp[lj->ncmp++] = 0;
        } else {
            for (int i = 0; i < nwant; i++)
                lj->cmp[lj->ncmp++] = (uint16_t)slot[want[i]];
        }
    }
    free(freed);
    free(slot);
    free(last);
    free(order);
    free(want);
    free(cur_a);
    free(cur_b);
    free(leaf);
    tc_net_free(net);
}

typedef struct {
    const Enum *const *jobs;
    LutJob           *out;
    int               njobs;
    int               next;
    pthread_mutex_t   lock;
} LutWork;

static void *lut_worker(void *arg)
{
    LutWork *w = arg;
    for (;;) {
        pthread_mutex_lock(&w->lock);
        int i = w->next++;
        pthread_mutex_unlock(&w->lock);
        if (i >= w->njobs)
            break;
        const Enum *e = w->jobs[i];
        memset(&w->out[i], 0, sizeof w->out[i]);
        if (e->ticks != 1 || !e->a)
            continue;
        size_t n = e->a->ninputs;
        int *in_map = tc_xcalloc(n + 1, sizeof *in_map);
        int *out_map = tc_xcalloc(e->a->noutputs + 1, sizeof *out_map);
        char err[256];
        if (tc_enum_prepare(e, in_map, out_map, err, sizeof err) && e->parts == 1)
            lut_job(e, in_map, out_map, &w->out[i]);
        free(in_map);
        free(out_map);
    }
    return NULL;
}

static void map_jobs(const Enum *const *jobs, int njobs, LutJob *out)
{
    LutWork w = {jobs, out, njobs, 0, PTHREAD_MUTEX_INITIALIZER};
    int threads = 16;
    if (threads > njobs)
        threads = njobs;
    pthread_t tid[16];
    for (int t = 0; t < threads; t++)
        pthread_create(&tid[t], NULL, lut_worker, &w);
    for (int t = 0; t < threads; t++)
        pthread_join(tid[t], NULL);
}

static int pack_job(Pack *pk, const Enum *e, const LutJob *lj, char *err, size_t errlen)
{
    const Program *a = e->a, *b = e->b;
    size_t n = a->ninputs;
    int *in_map = tc_xcalloc(n + 1, sizeof *in_map);
    int *out_map = tc_xcalloc(a->noutputs + 1, sizeof *out_map);
    int ok = 0;
    if (!tc_enum_prepare(e, in_map, out_map, err, errlen))
        goto done;
    if (e->parts != 1) {
        tc_fail(err, errlen, "the batched engine runs whole jobs, not --part shares");
        goto done;
    }
    if (e->ticks > 255) {
        tc_fail(err, errlen, "the batched engine runs at most 255 ticks");
        goto done;
    }
    unsigned slots = a->ncells + (e->mode == EN_EQUIV ? b->ncells : 0);
    const TcSpec *sp = (const TcSpec *)e->spec;
    if (e->mode == EN_VERIFY && sp->max_depth > 24) {
        tc_fail(err, errlen, "the batched engine evaluates specs nested at most 24 deep");
        goto done;
    }
    TcBatchJob J;
    memset(&J, 0, sizeof J);
    J.space = 1ull << n;
    if (lj && lj->ok) {
        J.words = (J.space + 31) / 32;
        J.mode = (uint8_t)e->mode;
        J.ticks = 1;
        J.lut = 1;
        J.slots = (uint16_t)lj->slots;
        J.one_a = CELL_ONE;
        J.code_a = (uint32_t)(pk->luts.n / 4);
        J.nb_a = (uint32_t)lj->nops;
        vpush(&pk->luts, lj->ops, (size_t)lj->nops * 4);
        J.lists = (uint32_t)pk->lists.n;
        J.n_in = (uint16_t)n;
        for (size_t k = 0; k < n; k++) {
            uint16_t s2[2] = {lj->in_slot[k], 0};
            vpush(&pk->lists, s2, 2);
        }
        vpush(&pk->lists, lj->cmp, (size_t)lj->ncmp);
        J.n_cmp = (uint16_t)(e->mode == EN_EQUIV ? lj->ncmp / 2
                             : e->mode == EN_SEARCH ? lj->ncmp / 2 : lj->ncmp);
        if (e->mode == EN_VERIFY) {
            J.rpn = (uint32_t)pk->rpn.n;
            J.nrpn = (uint16_t)sp->nrpn;
            for (int i = 0; i < sp->nrpn; i++) {
                TcBatchRpn it = {(uint32_t)sp->rpn[i].op, 0, sp->rpn[i].v};
                vpush(&pk->rpn, &it, 1);
            }
            J.vars = (uint32_t)pk->vars.n;
            J.nvars = (uint16_t)sp->nvars;
            for (int k = 0; k < sp->nvars; k++) {
                uint8_t d[65];
                memset(d, 0, sizeof d);
                d[0] = (uint8_t)sp->var_bits[k];
                for (int bit = 0; bit < sp->var_bits[k]; bit++)
                    d[1 + bit] = (uint8_t)sp->var_pos[k][bit];
                vpush(&pk->vars, d, 65);
            }
        }
        J.first_unit = pk->units;
        J.unit_words = pk->unit_words;
        J.units = (uint32_t)((J.words + J.unit_words - 1) / J.unit_words);
        pk->units += J.units;
        if ((int)J.slots > pk->slots)
            pk->slots = (int)J.slots;
        vpush(&pk->jobs, &J, 1);
        ok = 1;
        goto done;
    }
    if (slots > TC_BATCH_MAX_SLOTS) {
        tc_fail(err, errlen, "%u cells: more than the batched engine's %d slots", slots,
                TC_BATCH_MAX_SLOTS);
        goto done;
    }
    J.words = (J.space + 31) / 32;
    J.mode = (uint8_t)e->mode;
    J.ticks = (uint8_t)e->ticks;
    J.slots = (uint16_t)slots;
    J.one_a = CELL_ONE;
    unsigned bb = a->ncells;
    J.one_b = (uint16_t)(bb + CELL_ONE);
    J.code_a = pack_code(&pk->code, a, 0, &J.nb_a);
    if (e->mode == EN_EQUIV)
        J.code_b = pack_code(&pk->code, b, bb, &J.nb_b);
    J.lists = (uint32_t)pk->lists.n;
    J.n_in = (uint16_t)n;
    unsigned char *in_a = tc_xcalloc(a->ncells + 1, 1);
    unsigned char *in_b = tc_xcalloc((b ? b->ncells : 0) + 1, 1);
    for (size_t k = 0; k < n; k++) {
        uint16_t s[2] = {(uint16_t)a->inputs[k], 0};
        in_a[a->inputs[k]] = 1;
        if (e->mode == EN_EQUIV) {
            uint32_t cb = b->inputs[in_map[k]];
            s[1] = (uint16_t)(bb + cb);
            in_b[cb] = 1;
        }
        vpush(&pk->lists, s, 2);
    }
    clear_list(&pk->lists, a, 0, in_a, &J.n_zero);
    if (e->mode == EN_EQUIV)
        clear_list(&pk->lists, b, bb, in_b, &J.n_zero);
    free(in_a);
    free(in_b);
    if (e->mode == EN_EQUIV) {
        for (size_t o = 0; o < a->noutputs; o++) {
            uint16_t s[2] = {(uint16_t)a->outputs[o], (uint16_t)(bb + b->outputs[out_map[o]])};
            vpush(&pk->lists, s, 2);
        }
        J.n_cmp = (uint16_t)a->noutputs;
    } else if (e->mode == EN_SEARCH) {
        uint64_t target = cuda_spec_value(e->spec, 0);
        for (int i = 0; i < sp->width; i++) {
            uint16_t s[2] = {(uint16_t)sp->out[i], (uint16_t)((target >> i) & 1)};
            vpush(&pk->lists, s, 2);
        }
        J.n_cmp = (uint16_t)sp->width;
    } else {
        for (int i = 0; i < sp->width; i++) {
            uint16_t s = (uint16_t)sp->out[i];
            vpush(&pk->lists, &s, 1);
        }
        J.n_cmp = (uint16_t)sp->width;
        J.rpn = (uint32_t)pk->rpn.n;
        J.nrpn = (uint16_t)sp->nrpn;
        for (int i = 0; i < sp->nrpn; i++) {
            TcBatchRpn it = {(uint32_t)sp->rpn[i].op, 0, sp->rpn[i].v};
            vpush(&pk->rpn, &it, 1);
        }
        J.vars = (uint32_t)pk->vars.n;
        J.nvars = (uint16_t)sp->nvars;
        for (int k = 0; k < sp->nvars; k++) {
            uint8_t d[65];
            memset(d, 0, sizeof d);
            d[0] = (uint8_t)sp->var_bits[k];
            for (int bit = 0; bit < sp->var_bits[k]; bit++)
                d[1 + bit] = (uint8_t)sp->var_pos[k][bit];
            vpush(&pk->vars, d, 65);
        }
    }
    J.first_unit = pk->units;
    J.unit_words = pk->unit_words;
    J.units = (uint32_t)((J.words + J.unit_words - 1) / J.unit_words);
    pk->units += J.units;
    if ((int)slots > pk->slots)
        pk->slots = (int)slots;
    vpush(&pk->jobs, &J, 1);
    ok = 1;
done:
    free(in_map);
    free(out_map);
    return ok;
}

/* ---- waves: a set of jobs packed, launched on a stream, finished job by job ----------------- */

/* Mapped host buffers for waves, kept for reuse.  cudaFreeHost waits until every kernel on the
   device has finished (measured on GB300: 305 ms while a 305 ms kernel ran on another stream,
   where cudaHostAlloc took 1 ms), so freeing a finished wave's buffer would hold the serving loop
   until the other waves in flight are done, and no new wave would start meanwhile.  A finished
   wave's buffer goes back to the pool instead; tc_wave_pool_trim frees the pool once the device
   is idle. */
#define HOST_POOL 32
static struct {
    void  *p;
    size_t bytes;
    int    busy;
} host_pool[HOST_POOL];
static pthread_mutex_t host_pool_lock = PTHREAD_MUTEX_INITIALIZER;

/* A mapped buffer of at least `bytes`; *pooled = 0 when the pool is full (freed directly) */
static int host_get(void **p, size_t bytes, int *pooled, char *err, size_t errlen)
{
    pthread_mutex_lock(&host_pool_lock);
    int best = -1;
    for (int i = 0; i < HOST_POOL; i++)
        if (host_pool[i].p && !host_pool[i].busy && host_pool[i].bytes >= bytes &&
            (best < 0 || host_pool[i].bytes < host_pool[best].bytes))
            best = i;
    if (best >= 0) {
        host_pool[best].busy = 1;
        *p = host_pool[best].p;
        *pooled = 1;
        pthread_mutex_unlock(&host_pool_lock);
        return 1;
    }
    int empty = -1;
    for (int i = 0; i < HOST_POOL && empty < 0; i++)
        if (!host_pool[i].p)
            empty = i;
    size_t cap = bytes + bytes / 4 + ((size_t)1 << 20);  /* room for a somewhat larger wave */
    int ok = tc_cu_check(cudaHostAlloc(p, cap, cudaHostAllocMapped), "cudaHostAlloc", err, errlen);
    *pooled = ok && empty >= 0;
    if (*pooled) {
        host_pool[empty].p = *p;
        host_pool[empty].bytes = cap;
        host_pool[empty].busy = 1;
    }
    pthread_mutex_unlock(&host_pool_lock);
    return ok;
}

static void host_put(void *p, int pooled)
{
    if (!pooled) {
        cudaFreeHost(p);
        return;
    }
    pthread_mutex_lock(&host_pool_lock);
    for (int i = 0; i < HOST_POOL; i++)
        if (host_pool[i].p == p)
            host_pool[i].busy = 0;
    pthread_mutex_unlock(&host_pool_lock);
}

/* Frees the pool's idle buffers (each cudaFreeHost waits for the device to be idle). */
void tc_wave_pool_trim(void)
{
    pthread_mutex_lock(&host_pool_lock);
    for (int i = 0; i < HOST_POOL; i++)
        if (host_pool[i].p && !host_pool[i].busy) {
            cudaFreeHost(host_pool[i].p);
            host_pool[i].p = NULL;
            host_pool[i].bytes = 0;
        }
    pthread_mutex_unlock(&host_pool_lock);
}

struct TcWave {
    int                 njobs;
    const Enum        **jobs;       /* the wave's own copy: a caller may reuse its array */
    Pack                pk;
    uint32_t           *unit_job;
    void               *dev;        /* one device allocation for everything */
    void               *host;       /* one mapped host buffer: unit lists, results, flags */
    int                 host_pooled;
    unsigned long long *h_uhits, *h_hits;
    uint32_t           *h_ucount;
    volatile uint32_t  *h_done;
    cudaStream_t        stream;
    cudaEvent_t         ev0, ev1;
    int                 grid, launched;
    size_t              dev_bytes;
};

static size_t align256(size_t n)
{
    return (n + 255) & ~(size_t)255;
}

/* Blocks of the interpreter an SM holds when a block needs `slots` slots (shared memory is the
   limit; 16 blocks of 128 threads fill an SM). */
static int blocks_per_sm(int slots)
{
    int b = (int)(233472 / ((size_t)slots * TC_BATCH_BLOCK * 4 + 1024));
    return b < 1 ? 1 : b > 16 ? 16 : b;
}

/* Gives the jobs' units their launch order: jobs grouped by how many blocks per SM their slots
   allow (fewest slots first), a group too small to fill the GPU about twice merged into the
   next; within a group, job order. */
static void order_units(Pack *pk)
{
    TcBatchJob *J = pk->jobs.p;
    int n = (int)pk->jobs.n, sms = tc_engine.sms > 0 ? tc_engine.sms : 152;
    uint32_t units_at[17] = {0};
    for (int i = 0; i < n; i++)
        units_at[blocks_per_sm(J[i].slots)] += J[i].units;
    /* classes from 16 blocks per SM down to 1; small ones join the next */
    int cls_of[17], nclass = 0;
    uint32_t pending = 0;
    for (int b = 16; b >= 1; b--) {
        cls_of[b] = nclass;
        pending += units_at[b];
        if (pending && (pending >= (uint32_t)(2 * sms * b) || b == 1)) {
            nclass++;
            pending = 0;
        }
    }
    if (pending || !nclass)
        nclass++;
    for (int b = 1; b <= 16; b++)
        if (cls_of[b] >= nclass)
            cls_of[b] = nclass - 1;
    /* first units, class by class */
    uint32_t at = 0;
    for (int c = 0; c < nclass; c++) {
        pk->class_slots[c] = 1;
        for (int i = 0; i < n; i++) {
            int b = blocks_per_sm(J[i].slots);
            if (cls_of[b] != c)
                continue;
            J[i].first_unit = at;
            at += J[i].units;
            if (J[i].slots > pk->class_slots[c])
                pk->class_slots[c] = J[i].slots;
        }
        pk->class_end[c] = at;
    }
    pk->nclass = nclass;
}

/* Maps and packs the jobs (no device work yet). */
int tc_wave_prepare(TcWave **out, const Enum *const *jobs, int njobs, char *err, size_t errlen)
{
    TcWave *w = tc_xcalloc(1, sizeof *w);
    w->njobs = njobs;
    w->jobs = tc_xmalloc(((size_t)njobs + 1) * sizeof *w->jobs);
    memcpy(w->jobs, jobs, (size_t)njobs * sizeof *w->jobs);
    w->pk.jobs.elem = sizeof(TcBatchJob);
    w->pk.code.elem = 8;
    w->pk.luts.elem = 4;
    w->pk.lists.elem = 2;
    w->pk.rpn.elem = sizeof(TcBatchRpn);
    w->pk.vars.elem = 1;
    /* units of TC_BATCH_UNIT_WORDS, or smaller for a wave too small to give every resident block
       of the GPU a few units (a served wave of light jobs): its units would run one after another
       in a few blocks while the rest of the GPU waits */
    double words = 0;
    for (int i = 0; i < njobs; i++)
        words += jobs[i]->a->ninputs < 64 ? ldexp(1.0, (int)jobs[i]->a->ninputs) / 32 : 1e30;
    double want = 4.0 * (tc_engine.sms > 0 ? tc_engine.sms : 152) * 8;  /* units */
    w->pk.unit_words = TC_BATCH_UNIT_WORDS;
    while (w->pk.unit_words > TC_BATCH_UNIT_WORDS_MIN && words / w->pk.unit_words < want)
        w->pk.unit_words /= 2;
    LutJob *lj = tc_xcalloc((size_t)njobs + 1, sizeof *lj);
    map_jobs(jobs, njobs, lj);
    int ok = 1;
    for (int i = 0; i < njobs && ok; i++) {
        char e2[400];
        if (!pack_job(&w->pk, jobs[i], &lj[i], e2, sizeof e2)) {
            tc_fail(err, errlen, "job %d: %s", i, e2);
            ok = 0;
        }
    }
    for (int i = 0; i < njobs; i++) {
        free(lj[i].ops);
        free(lj[i].in_slot);
        free(lj[i].cmp);
    }
    free(lj);
    if (!ok) {
        tc_wave_free(w);
        return 0;
    }
    order_units(&w->pk);
    w->unit_job = tc_xmalloc(((size_t)w->pk.units + 1) * sizeof *w->unit_job);
    const TcBatchJob *J = w->pk.jobs.p;
    for (int i = 0; i < njobs; i++)
        for (uint32_t u = 0; u < J[i].units; u++)
            w->unit_job[J[i].first_unit + u] = (uint32_t)i;
    *out = w;
    return 1;
}

size_t tc_wave_bytes(const TcWave *w)
{
    const Pack *pk = &w->pk;
    return align256(pk->jobs.n * pk->jobs.elem) + align256(pk->code.n * 8) +
           align256(pk->luts.n * 4) + align256(pk->lists.n * 2) +
           align256(pk->rpn.n * pk->rpn.elem) + align256(pk->vars.n) +
           align256((size_t)pk->units * 4) + 256 + align256((size_t)w->njobs * 8) +
           align256((size_t)w->njobs * 4);
}

/* Uploads and launches on `stream`; the grid takes `share` of the GPU's resident blocks. */
int tc_wave_launch(TcWave *w, cudaStream_t stream, double share, char *err, size_t errlen)
{
    Pack *pk = &w->pk;
    int n = w->njobs;
    size_t off[10], at = 0;
    size_t sizes[10] = {pk->jobs.n * pk->jobs.elem, pk->code.n * 8, pk->luts.n * 4,
                        pk->lists.n * 2, pk->rpn.n * pk->rpn.elem, pk->vars.n,
                        (size_t)pk->units * 4, MAX_CLASSES * 4, (size_t)n * 8, (size_t)n * 4};
    for (int i = 0; i < 10; i++) {
        off[i] = at;
        at += align256(sizes[i] ? sizes[i] : 1);
    }
    w->dev_bytes = at;
    size_t hsz[4] = {(size_t)pk->units * TC_BATCH_SHOW * 8, (size_t)pk->units * 4,
                     (size_t)n * 8, (size_t)n * 4};
    size_t hoff[4], hat = 0;
    for (int i = 0; i < 4; i++) {
        hoff[i] = hat;
        hat += align256(hsz[i] ? hsz[i] : 1);
    }
    w->stream = stream;
    if (!tc_cu_check(cudaMallocAsync(&w->dev, at, stream), "cudaMallocAsync", err, errlen) ||
        !host_get(&w->host, hat, &w->host_pooled, err, errlen))
        return 0;
    memset(w->host, 0, hat);
    char *h = w->host;
    w->h_uhits = (unsigned long long *)(h + hoff[0]);
    w->h_ucount = (uint32_t *)(h + hoff[1]);
    w->h_hits = (unsigned long long *)(h + hoff[2]);
    w->h_done = (volatile uint32_t *)(h + hoff[3]);
    char *hd;
    if (!tc_cu_check(cudaHostGetDevicePointer((void **)&hd, w->host, 0), "mapped memory", err,
                     errlen))
        return 0;
    char *d = w->dev;
    const void *src[7] = {pk->jobs.p, pk->code.p, pk->luts.p, pk->lists.p, pk->rpn.p, pk->vars.p,
                          w->unit_job};
    for (int i = 0; i < 7; i++)
        if (sizes[i] && !tc_cu_check(cudaMemcpyAsync(d + off[i], src[i], sizes[i],
                                                     cudaMemcpyHostToDevice, stream),
                                     "upload", err, errlen))
            return 0;
    /* units left per job */
    uint32_t *rem = tc_xmalloc((size_t)n * 4 + 4);
    const TcBatchJob *J = pk->jobs.p;
    for (int i = 0; i < n; i++)
        rem[i] = J[i].units;
    int ok = tc_cu_check(cudaMemcpyAsync(d + off[9], rem, (size_t)n * 4, cudaMemcpyHostToDevice,
                                         stream), "upload", err, errlen) &&
             tc_cu_check(cudaMemsetAsync(d + off[7], 0, MAX_CLASSES * 4, stream), "memset", err,
                         errlen) &&
             tc_cu_check(cudaMemsetAsync(d + off[8], 0, (size_t)n * 8, stream), "memset", err,
                         errlen);
    /* the host buffer must outlive the asynchronous copy: wait for it */
    if (ok)
        ok = tc_cu_check(cudaStreamSynchronize(stream), "upload", err, errlen);
    free(rem);
    if (!ok)
        return 0;
    struct TcBatchDev dv = {(const TcBatchJob *)(d + off[0]), (const uint64_t *)(d + off[1]),
                            (const uint32_t *)(d + off[2]), (const uint16_t *)(d + off[3]),
                            (const TcBatchRpn *)(d + off[4]), (const uint8_t *)(d + off[5]),
                            (const uint32_t *)(d + off[6]), 0, pk->units, (uint32_t *)(d + off[7]),
                            (unsigned long long *)(d + off[8]),
                            (unsigned long long *)(hd + hoff[0]), (uint32_t *)(hd + hoff[1]),
                            (uint32_t *)(d + off[9]), (unsigned long long *)(hd + hoff[2]),
                            (uint32_t *)(hd + hoff[3])};
    if (!tc_cu_check(cudaEventCreate(&w->ev0), "event", err, errlen) ||
        !tc_cu_check(cudaEventCreate(&w->ev1), "event", err, errlen) ||
        !tc_cu_check(cudaEventRecord(w->ev0, stream), "event", err, errlen))
        return 0;
    /* one launch per class, each with its own counter and slot count */
    w->grid = 0;
    for (int c = 0; c < pk->nclass; c++) {
        int grid = 0;
        dv.unit_base = c ? pk->class_end[c - 1] : 0;
        dv.nunits = pk->class_end[c];
        dv.next_unit = (uint32_t *)(d + off[7]) + c;
        if (dv.nunits == dv.unit_base)
            continue;
        if (!tc_batch_launch(&dv, pk->class_slots[c], stream, share, &grid, err, errlen))
            return 0;
        if (grid > w->grid)
            w->grid = grid;
    }
    if (!tc_cu_check(cudaEventRecord(w->ev1, stream), "event", err, errlen))
        return 0;
    w->launched = 1;
    return 1;
}

/* The flag is read with acquire order: on a weakly ordered host (Grace is aarch64) the reads of
   the job's counts and hit lists in host-mapped memory that tc_wave_result makes after it must
   not be satisfied before the flag was seen set (the kernel fences them before the flag). */
int tc_wave_job_done(const TcWave *w, int i)
{
    return __atomic_load_n((const uint32_t *)&w->h_done[i], __ATOMIC_ACQUIRE) != 0;
}

/* 1 when the wave's kernel has finished (0 still running, -1 error) */
int tc_wave_finished(const TcWave *w)
{
    cudaError_t e = cudaEventQuery(w->ev1);
    return e == cudaSuccess ? 1 : e == cudaErrorNotReady ? 0 : -1;
}

float tc_wave_ms(const TcWave *w)
{
    float ms = 0;
    cudaEventElapsedTime(&ms, w->ev0, w->ev1);
    return ms;
}

/* Job i's result, valid once tc_wave_job_done(w, i). */
void tc_wave_result(const TcWave *w, int i, EnumResult *r)
{
    const TcBatchJob *J = w->pk.jobs.p;
    const Enum *e = w->jobs[i];
    memset(r, 0, sizeof *r);
    r->space = J[i].space;
    r->tried = J[i].space;
    uint64_t passes = (J[i].space + 511) / 512;
    r->ops = passes * 512 * e->ticks * (e->a->len + (e->mode == EN_EQUIV ? e->b->len : 0));
    r->hits = w->h_hits[i];
    r->threads = w->grid * TC_BATCH_BLOCK;
    for (uint32_t u = 0; u < J[i].units && r->nhit < EN_SHOW && r->hits; u++) {
        uint32_t c = w->h_ucount[J[i].first_unit + u];
        for (uint32_t h = 0; h < c; h++)
            cuda_enum_add_hit(r, w->h_uhits[(size_t)(J[i].first_unit + u) * TC_BATCH_SHOW + h]);
    }
}

int tc_wave_njobs(const TcWave *w)
{
    return w->njobs;
}

/* Shared-memory slots job i uses (each is 4 bytes per thread). */
int tc_wave_job_slots(const TcWave *w, int i)
{
    return ((const TcBatchJob *)w->pk.jobs.p)[i].slots;
}

void tc_wave_free(TcWave *w)
{
    if (!w)
        return;
    if (w->dev)
        cudaFreeAsync(w->dev, w->stream);
    if (w->host) {
        if (w->launched)
            cudaEventSynchronize(w->ev1);
        host_put(w->host, w->host_pooled);
    }
    if (w->ev0)
        cudaEventDestroy(w->ev0);
    if (w->ev1)
        cudaEventDestroy(w->ev1);
    free(w->unit_job);
    free(w->jobs);
    free(w->pk.jobs.p);
    free(w->pk.code.p);
    free(w->pk.luts.p);
    free(w->pk.lists.p);
    free(w->pk.rpn.p);
    free(w->pk.vars.p);
    free(w);
}

/* ---- a batch: every job at once ---------------------------------------------------------------

   cuda_batch_run hands the jobs to the serving loop as if they all arrived at the start.  A plan
   (plan() below) sends to generated code the jobs that save the most interpreter time per second
   of compiling, as long as their compiles, spread over the host's cores, end well before the
   interpreter is through with the rest; a job whose kernel is cached already goes there whenever
   its work is worth a launch.  The interpreter's jobs run as persistent launches from a device
   work queue, in waves of a quarter of the batch on two streams (the GPU starts once the first
   quarter is packed) with 90 % of the blocks; the compiles start once the first wave is out and
   the remaining blocks run the compiled jobs as they come; jobs still waiting for a compile
   thread when the interpreter runs out of work go back to it.  Results do not depend on the
   route: both engines enumerate the whole job. */

int    tc_serve_batch(const Enum *const *jobs, int njobs, const CudaServeOpts *opts,
                      const signed char *route, int first_wave, double *finish,
                      EnumResult *results, int *engine_used, char *err, size_t errlen);
double tc_route_compile_s(const Enum *e, double instrs);
extern double tc_serve_last_wave_at, tc_serve_last_compile_busy, tc_serve_last_compile_load,
    tc_serve_last_loop_end;
extern int    tc_serve_last_routed, tc_serve_last_taken_back;
double tc_route_compiled_s(const Enum *e, double work);

/* The interpreter's rate on a batch with most of the GPU (1.39e14 NAND/STO lane-ops/s measured
   on the 4,096-job batch alone; host packing and a 90 % share of the blocks beside compiled
   jobs bring it to about this). */
#define BATCH_RATE_INTERP 1.1e14
/* the interpreter's share of the GPU's resident blocks when jobs also run compiled */
double tc_batch_share = 0.9;
#define BATCH_SHARE tc_batch_share

static CudaBatchStats last_batch;

/* compile threads of a batch (0: the host's cores less two) */
int tc_batch_threads = 0;
/* the share of the interpreter's time the plan fills with compiling (see plan()) */
double tc_batch_plan_share = 0.7;

typedef struct {
    double work, instrs, compile_s, compiled_s, gain;
    int    i;
} Planned;

static int by_gain(const void *x, const void *y)
{
    const Planned *a = x, *b = y;
    return a->gain < b->gain ? 1 : a->gain > b->gain ? -1 : a->i - b->i;
}

/* The batch's plan: jobs by the interpreter time they would save per second of compiling (a
   cached kernel costs none), taken for generated code while the compiling of those taken, spread
   over the compile threads, ends before the interpreter is through with the jobs it keeps; cached
   jobs whenever their work is worth a launch.  The compiles then cost no time of the batch. */
static void plan(Planned *p, int n, int threads, signed char *route)
{
    double interp = 0, compile = 0;
    for (int k = 0; k < n; k++)
        interp += p[k].work / BATCH_RATE_INTERP;
    for (int k = 0; k < n; k++) {
        double saved = p[k].work / BATCH_RATE_INTERP - p[k].compiled_s;
        double c = p[k].compile_s / threads;
        /* 70 % of the interpreter's time: compiles start once its first wave is packed and run
           slower than modelled when every core compiles; jobs still queued when the
           interpreter runs out go back to it (measured on the 4,096-job batch with PTX builds:
           0.5 3,463, 0.7 3,793, 0.9 3,680 jobs/s) */
        route[k] = saved > 0 && (c == 0 || compile + c <= tc_batch_plan_share *
                                                              (interp - p[k].work / BATCH_RATE_INTERP));
        if (route[k]) {
            compile += c;
            interp -= p[k].work / BATCH_RATE_INTERP;
        }
    }
}

int cuda_batch_run(const Enum *const *jobs, int njobs, EnumResult *results, char *err,
                   size_t errlen)
{
    memset(&last_batch, 0, sizeof last_batch);
    if (njobs <= 0)
        return 1;
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    double t0 = tc_now();
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int threads = tc_batch_threads > 0 ? tc_batch_threads
                  : cores > 3 ? (int)cores - 2 : 1;  /* the host loop and the CUDA runtime keep a core */
    Planned *p = tc_xmalloc((size_t)njobs * sizeof *p);
    for (int i = 0; i < njobs; i++) {
        const Enum *e = jobs[i];
        p[i].i = i;
        p[i].instrs = (double)e->a->len + (e->mode == EN_EQUIV && e->b ? (double)e->b->len : 0);
        p[i].work = (e->a->ninputs < 64 ? (double)(1ull << e->a->ninputs) : 0) * e->ticks *
                    p[i].instrs;
        /* a job whose GPU time saved would not pay for a launch stays on the interpreter
           whatever the cache holds: no need to look (the look hashes both programs) */
        p[i].compiled_s = tc_route_compiled_s(e, p[i].work);
        int worth = p[i].work / BATCH_RATE_INTERP - p[i].compiled_s > 0;
        p[i].compile_s = e->parts == 1 && worth ? tc_route_compile_s(e, p[i].instrs) : 1e30;
        p[i].gain = p[i].work / (p[i].compile_s > 0 ? p[i].compile_s : 1e-9);
    }
    qsort(p, (size_t)njobs, sizeof *p, by_gain);
    signed char *route = tc_xcalloc((size_t)njobs, 1);
    plan(p, njobs, threads, route);
    const Enum **order = tc_xmalloc((size_t)njobs * sizeof *order);
    for (int k = 0; k < njobs; k++)
        order[k] = jobs[p[k].i];
    double *finish = tc_xcalloc((size_t)njobs, sizeof *finish);
    EnumResult *res = tc_xcalloc((size_t)njobs, sizeof *res);
    int *engine = tc_xcalloc((size_t)njobs, sizeof *engine), any = 0;
    for (int k = 0; k < njobs; k++)
        any |= route[k];
    CudaServeOpts o;
    memset(&o, 0, sizeof o);
    /* waves of a quarter on two streams: the GPU starts once the first quarter is packed */
    o.streams = 2;
    o.max_inflight_jobs = njobs;
    o.max_wave_jobs = njobs >= 256 ? (njobs + 3) / 4 : njobs;
    o.max_device_bytes = (size_t)64 << 30;
    o.share = any ? BATCH_SHARE : 1.0;
    o.compile_threads = any ? threads : -1;
    o.compiled_slots = 8;
    o.route = any ? CUDA_SERVE_AUTO : CUDA_SERVE_INTERPRETER;
    /* a first wave of a sixteenth: the GPU, and the held compiles, start once it is packed */
    int first = njobs >= 1024 ? njobs / 16 : 0;
    int ok = tc_serve_batch(order, njobs, &o, route, first, finish, res, engine, err, errlen);
    double wall = tc_now() - t0;
    if (ok) {
        for (int k = 0; k < njobs; k++) {
            results[p[k].i] = res[k];
            results[p[k].i].seconds = wall;
            last_batch.compiled += engine[k];
        }
        last_batch.jobs = njobs;
        last_batch.interpreted = njobs - last_batch.compiled;
        last_batch.compile_threads = any ? threads : 0;
        last_batch.seconds = wall;
        last_batch.interpreter_start = tc_serve_last_wave_at;
        last_batch.planned = tc_serve_last_routed;
        last_batch.taken_back = tc_serve_last_taken_back;
        last_batch.compile_busy = tc_serve_last_compile_busy;
        last_batch.compile_load = tc_serve_last_compile_load;
        last_batch.loop_end = tc_serve_last_loop_end;
        double last_interp = 0, last_compiled = 0;
        for (int k = 0; k < njobs; k++) {
            double *at = engine[k] ? &last_compiled : &last_interp;
            if (finish[k] > *at)
                *at = finish[k];
        }
        last_batch.interpreter_end = last_interp;
        last_batch.compiled_end = last_compiled;
    }
    free(p);
    free(route);
    free(order);
    free(finish);
    free(res);
    free(engine);
    return ok;
}

/* cuda_batch_prepare: compile threads take groups of up to four jobs in turn */
typedef struct {
    const Enum *const *jobs;
    const int         *ids;
    TcEnumJob         *prep;
    int                n, next, failed;
    double             busy;
    char               err[512];
    pthread_mutex_t    mu;
} Prepare;

static void *prepare_worker(void *arg)
{
    Prepare *w = arg;
    for (;;) {
        pthread_mutex_lock(&w->mu);
        int k0 = w->next, n = w->n - k0 < 4 ? w->n - k0 : 4;
        w->next += n > 0 ? n : 0;
        int stop = n <= 0 || w->failed;
        pthread_mutex_unlock(&w->mu);
        if (stop)
            return NULL;
        const Enum *es[4];
        TcEnumJob *js[4];
        for (int i = 0; i < n; i++) {
            es[i] = w->jobs[w->ids[k0 + i]];
            js[i] = &w->prep[k0 + i];
        }
        char e2[512];
        double t0 = tc_now();
        int ok = tc_enum_jobs_build(es, js, n, TC_BUILD_SERVE, e2, sizeof e2);
        pthread_mutex_lock(&w->mu);
        w->busy += tc_now() - t0;
        if (!ok && !w->failed) {
            w->failed = 1;
            snprintf(w->err, sizeof w->err, "%s", e2);
        }
        pthread_mutex_unlock(&w->mu);
    }
}

double tc_batch_last_prepare_busy;

int cuda_batch_prepare(const Enum *const *jobs, int njobs, int *prepared, char *err,
                       size_t errlen)
{
    if (prepared)
        *prepared = 0;
    if (njobs <= 0)
        return 1;
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    long cores = sysconf(_SC_NPROCESSORS_ONLN);
    int threads = tc_batch_threads > 0 ? tc_batch_threads : cores > 3 ? (int)cores - 2 : 1;
    if (threads > 64)
        threads = 64;
    Prepare w;
    memset(&w, 0, sizeof w);
    pthread_mutex_init(&w.mu, NULL);
    int *ids = tc_xmalloc((size_t)njobs * sizeof *ids);
    /* the jobs a batch could send to generated code: whole spaces whose work pays for a launch */
    for (int i = 0; i < njobs; i++) {
        const Enum *e = jobs[i];
        double instrs = (double)e->a->len + (e->mode == EN_EQUIV && e->b ? (double)e->b->len : 0);
        double work = (e->a->ninputs < 64 ? (double)(1ull << e->a->ninputs) : 0) * e->ticks *
                      instrs;
        if (e->parts == 1 && work / BATCH_RATE_INTERP - tc_route_compiled_s(e, work) > 0)
            ids[w.n++] = i;
    }
    w.jobs = jobs;
    w.ids = ids;
    w.prep = tc_xcalloc((size_t)w.n + 1, sizeof *w.prep);
    pthread_t tid[64];
    int nt = 0;
    for (; nt < threads && nt * 4 < w.n; nt++)
        if (pthread_create(&tid[nt], NULL, prepare_worker, &w) != 0)
            break;
    if (nt == 0)
        prepare_worker(&w);
    for (int i = 0; i < nt; i++)
        pthread_join(tid[i], NULL);
    int ok = !w.failed;
    if (!ok)
        tc_fail(err, errlen, "%s", w.err);
    /* every build loaded: the first load of a module waits for the device's running work */
    for (int k = 0; k < w.n; k++) {
        if (ok && w.prep[k].pending)
            ok = tc_enum_job_load(jobs[ids[k]], &w.prep[k], err, errlen);
        else
            tc_enum_job_drop(&w.prep[k]);
    }
    if (ok && prepared)
        *prepared = w.n;
    tc_batch_last_prepare_busy = w.busy;
    pthread_mutex_destroy(&w.mu);
    free(w.prep);
    free(ids);
    return ok;
}

int cuda_batch_stats(CudaBatchStats *s)
{
    *s = last_batch;
    return last_batch.jobs > 0;
}
