// The superoptimizer on the GPU: iterative deepening over the budget.  For each budget the top of
// the search tree is expanded breadth-first on the device, one kernel per level, until the level
// holds enough states to keep every thread busy; then every GPU thread runs an explicit-stack
// depth-first search of frontier subtrees taken from a work queue.  The search model and its
// pruning are in super_search.cuh; the first thread to reach the goal records its state and
// raises a flag the others poll, as the reference's threads share one stop flag
// (src/super.c:770-896).
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "engine.h"
#include "super_search.cuh"

#define DEV_LEVELS 44      // deepest level a device search reaches (budgets up to 44)
#define POLL 1024          // nodes between looks at the stop flag
#define FRONT_PER_THREAD 16  // frontier states per search thread, for the work queue's balance
#define FRONT_MAX (8u << 20) // states one frontier level may hold (776 B each: 6.5 GB)

// ---- the top of the tree, breadth-first ---------------------------------------------------------

struct SpExpand {
    const SpSpec *spec;
    const SpState *in;
    unsigned long long nin;
    SpState *out;               // null: count only
    unsigned long long *count;  // children kept (not pruned, not the goal)
    unsigned long long *nodes;
    int *found;
    SpState *sol;
    int budget;
};

// The children of one state, in the order the reference's node() visits them (src/super.c:641-716): every operand
// the state's NAND may read, then every subset of the outputs the new RR value writes.  Each child
// counts as a node; a goal is recorded, a pruned child dropped, the rest kept: counted, or written
// to out[base ...] in visiting order.
__device__ unsigned long long expand_one(const SpSpec *sp, SpState *x, int budget,
                                         SpState *out, unsigned long long base,
                                         unsigned long long *nodes, int *found, SpState *sol)
{
    SpCand cand[SP_CANDS];
    const int m = sp_build(sp, x, cand);
    unsigned long long kept = 0;
    for (int i = 0; i < m; i++) {
        const uint32_t used = x->used;
        if (!sp_nand(sp, x, &cand[i], budget))
            continue;
        int8_t list[SP_CELLS];
        const int k = sp_hits(sp, x, list);
        for (int mask = 0; mask < (1 << k); mask++) {
            const uint32_t readable = x->readable, written = x->written;
            const int cost = x->cost;
            sp_write(sp, x, list, mask);
            if (nodes)
                (*nodes)++;
            const int a = sp_arrive(sp, x, budget);
            if (a == 2 && found) {
                if (atomicCAS(found, 0, 1) == 0)
                    *sol = *x;
            } else if (a == 0) {
                if (out)
                    out[base + kept] = *x;
                kept++;
            }
            x->readable = readable;
            x->written = written;
            x->cost = cost;
        }
        if (cand[i].kind == SK_LAZY)
            x->stored[cand[i].ref] = 0;
        x->cost -= 1 + cand[i].extra;
        x->n--;
        x->used = used;
    }
    return kept;
}

// One level: with out null, counts the children, the nodes and any goal; with out set, each
// thread counts its state's children again, takes a run of slots and writes them there.
__global__ void __launch_bounds__(128) tc_super_expand(SpExpand e)
{
    __shared__ SpSpec sp_s;
    if (threadIdx.x == 0)
        sp_s = *e.spec;
    __syncthreads();
    const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e.nin)
        return;
    SpState x = e.in[i];
    if (!e.out) {
        unsigned long long nodes = 0;
        const unsigned long long kept =
            expand_one(&sp_s, &x, e.budget, nullptr, 0, &nodes, e.found, e.sol);
        atomicAdd(e.nodes, nodes);
        if (kept)
            atomicAdd(e.count, kept);
        return;
    }
    const unsigned long long kept =
        expand_one(&sp_s, &x, e.budget, nullptr, 0, nullptr, nullptr, nullptr);
    if (!kept)
        return;
    const unsigned long long base = atomicAdd(e.count, kept);
    expand_one(&sp_s, &x, e.budget, e.out, base, nullptr, nullptr, nullptr);
}

// ---- device: depth-first search of one subtree -------------------------------------------------

// Raw operand sources: 0 ZERO, 1 ONE, 2 + c cell c, 18 + j RR value hist[j].
__device__ __forceinline__ int raw_cand(const SpSpec *sp, const SpState *x, int i, SpCand *c)
{
    if (i == 0) {
        c->v = 0; c->kind = SK_ZERO; c->extra = 0; c->ref = 0;
        return 1;
    }
    if (i == 1) {
        c->v = sp->mask; c->kind = SK_ONE; c->extra = 0; c->ref = 0;
        return 1;
    }
    if (i < 2 + SP_CELLS) {
        int cc = i - 2;
        if (cc >= sp->ncells || !((x->readable >> cc) & 1))
            return 0;
        int prev = sp->sym_prev[cc];
        if (prev >= 0 && !((x->used >> prev) & 1))
            return 0;
        c->v = sp_cell_value(sp, x, cc); c->kind = SK_CELL; c->extra = 0; c->ref = (int8_t)cc;
        return 1;
    }
    int j = i - 2 - SP_CELLS;
    if (j > x->n || (j == 0 && !x->def0))
        return 0;
    c->v = x->hist[j];
    c->kind = x->stored[j] ? SK_TEMP : SK_LAZY;
    c->extra = (uint8_t)!x->stored[j];
    c->ref = (int8_t)j;
    return 1;
}

// The operands of the node as a set of raw sources: one per value, the cheapest.
__device__ uint64_t survivors(const SpSpec *sp, const SpState *x)
{
    uint64_t keep = 0;
    uint64_t val[2 + SP_CELLS + DEV_LEVELS + 1];
    uint8_t extra[2 + SP_CELLS + DEV_LEVELS + 1];
    int idx[2 + SP_CELLS + DEV_LEVELS + 1], m = 0;
    int top = 2 + SP_CELLS + x->n;
    for (int i = 0; i <= top; i++) {
        SpCand c;
        if (!raw_cand(sp, x, i, &c))
            continue;
        int k = 0;
        while (k < m && val[k] != c.v)
            k++;
        if (k == m) {
            val[m] = c.v;
            extra[m] = c.extra;
            idx[m++] = i;
        } else if (c.extra < extra[k]) {
            extra[k] = c.extra;
            idx[k] = i;
        }
    }
    for (int k = 0; k < m; k++)
        keep |= 1ull << idx[k];
    return keep;
}

struct SpDev {
    const SpSpec *spec;
    const SpState *frontier;
    unsigned long long nfront;
    int budget;
    unsigned long long *next;
    int *found;
    SpState *sol;
    unsigned long long *nodes;
    ulonglong2 *tt;             // the transposition table, shared by every thread
    unsigned long long tt_mask;
    int tt_min_rem;             // states with fewer instructions left are not looked up
};

// Subtrees with fewer instructions left than this are searched again rather than looked up:
// a lookup is a random global-memory access and a key over every operand value.
extern "C" {
int tc_super_tt_min_rem = 4;
}

// ---- the transposition table ------------------------------------------------------------------
//
// States searched in full without a program, as the reference's per-thread table keeps them
// (src/super.c:408-418, 641-716): the same state is reached in many orders, and its future
// depends only on RR, the readable, written and used cells, and the values a NAND could read with
// what each costs.  Here one table serves every thread, and it is kept from budget to budget.  An
// entry is two 64-bit words: the state's first key, and its second key with the low byte
// replaced by the instructions that were left when it was searched; a state arriving with `rem`
// left is pruned when an entry holds both its keys and at least `rem`.  An entry torn between two
// writers matches only when both wrote this state (the rem is then a true one) or by a 120-bit
// coincidence, which the reference's 128-bit keys also rule out in practice.

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The state's keys (src/super.c:626-641): RR, the cell masks, and the operand values as a set.
__device__ void state_key(const SpSpec *sp, const SpState *x, uint64_t keep, uint64_t *k1,
                          uint64_t *k2)
{
    uint64_t a = mix64(x->hist[x->n] ^ (uint64_t)sp_rr_def(x) << 63), b = mix64(a + 0x1234567);
    const uint64_t f = (uint64_t)x->readable | (uint64_t)x->written << 21 |
                       (uint64_t)x->used << 42;
    a += mix64(f + 0x9E3779B97F4A7C15ull);
    b ^= mix64(f * 3 + 77);
    for (uint64_t rest = keep; rest; rest &= rest - 1) {
        SpCand c;
        raw_cand(sp, x, __ffsll((long long)rest) - 1, &c);
        const uint64_t v = c.v * 2 + c.extra;
        a += mix64(v + 0x51ED27);
        b += mix64(v * 0x2545F4914F6CDD1Dull + 0xABCDEF);
    }
    *k1 = a;
    *k2 = b;
}

__device__ __forceinline__ bool tt_seen(const SpDev &d, uint64_t k1, uint64_t k2, int rem)
{
    const ulonglong2 e = d.tt[k1 & d.tt_mask];
    return e.x == k1 && (e.y & ~0xFFull) == (k2 & ~0xFFull) && (int)(e.y & 0xFFull) >= rem;
}

__device__ __forceinline__ void tt_store(const SpDev &d, uint64_t k1, uint64_t k2, int rem)
{
    d.tt[k1 & d.tt_mask] = make_ulonglong2(k1, (k2 & ~0xFFull) | (uint64_t)rem);
}

__global__ void __launch_bounds__(128) tc_super_kernel(SpDev d)
{
    __shared__ SpSpec sp_s;
    if (threadIdx.x == 0)
        sp_s = *d.spec;
    __syncthreads();
    const SpSpec *sp = &sp_s;
    SpState x;
    uint64_t keep[DEV_LEVELS + 1];
    uint8_t ci[DEV_LEVELS + 1], k_at[DEV_LEVELS + 1];
    uint16_t wmask[DEV_LEVELS + 1];
    uint32_t w_readable[DEV_LEVELS + 1], w_written[DEV_LEVELS + 1], used_before[DEV_LEVELS + 1];
    int w_cost[DEV_LEVELS + 1];
    uint64_t key1[DEV_LEVELS + 1], key2[DEV_LEVELS + 1];
    int8_t key_rem[DEV_LEVELS + 1];  // rem of the node at this level, or -1: not in the table
    unsigned long long nodes = 0, polled = 0;
    const int budget = d.budget;
    for (;;) {
        const unsigned long long f = atomicAdd(d.next, 1ull);
        if (f >= d.nfront || *(volatile int *)d.found)
            break;
        x = d.frontier[f];
        const int n0 = x.n;
        int L = n0;
        keep[L] = survivors(sp, &x);
        ci[L] = 0;
        key_rem[L] = -1;
        bool expand = true;
        for (;;) {
            if (nodes - polled >= POLL) {
                polled = nodes;
                if (*(volatile int *)d.found)
                    break;
            }
            if (expand) {
                const uint64_t rest = keep[L] & (~0ull << ci[L]);
                if (!rest) {  // every operand tried at this level
                    if (L == n0)
                        break;
                    if (key_rem[L] >= 0)  // searched in full, nothing found
                        tt_store(d, key1[L], key2[L], key_rem[L]);
                    x.readable = w_readable[L];
                    x.written = w_written[L];
                    x.cost = w_cost[L];
                    wmask[L]++;
                    expand = false;
                    continue;
                }
                const int i = __ffsll((long long)rest) - 1;
                ci[L] = (uint8_t)(i + 1);
                SpCand c;
                raw_cand(sp, &x, i, &c);
                const uint32_t used = x.used;
                if (L + 1 > DEV_LEVELS || !sp_nand(sp, &x, &c, budget))
                    continue;
                L++;
                used_before[L] = used;
                int8_t list[SP_CELLS];
                k_at[L] = (uint8_t)sp_hits(sp, &x, list);
                wmask[L] = 0;
                expand = false;
                continue;
            }
            // the output writes after NAND L
            if (wmask[L] >= (1u << k_at[L])) {  // all tried: take the NAND back
                if (x.op_kind[L] == SK_LAZY)
                    x.stored[x.op_ref[L]] = 0;
                x.cost -= 1 + (x.op_kind[L] == SK_LAZY);
                x.used = used_before[L];
                x.n--;
                L--;
                expand = true;
                continue;
            }
            int8_t list[SP_CELLS];
            sp_hits(sp, &x, list);
            w_readable[L] = x.readable;
            w_written[L] = x.written;
            w_cost[L] = x.cost;
            sp_write(sp, &x, list, wmask[L]);
            nodes++;
            const int a = sp_arrive(sp, &x, budget);
            if (a == 2) {
                if (atomicCAS(d.found, 0, 1) == 0)
                    *d.sol = x;
                break;
            }
            if (a == 0) {
                keep[L] = survivors(sp, &x);
                ci[L] = 0;
                key_rem[L] = -1;
                const int rem = budget - x.cost;
                bool seen = false;
                if (rem >= d.tt_min_rem) {  // small subtrees: cheaper to search again
                    state_key(sp, &x, keep[L], &key1[L], &key2[L]);
                    seen = tt_seen(d, key1[L], key2[L], rem);
                    key_rem[L] = (int8_t)rem;
                }
                if (!seen) {
                    expand = true;
                    continue;
                }
                key_rem[L] = -1;  // searched before with at least this much left: nothing there
            }
            x.readable = w_readable[L];
            x.written = w_written[L];
            x.cost = w_cost[L];
            wmask[L]++;
        }
        if (*(volatile int *)d.found)
            break;
    }
    atomicAdd(d.nodes, nodes);
}

// ---- the driver ----------------------------------------------------------------------------------

// Grows *buf to hold n states.
static int reserve(SpState **buf, size_t *cap, size_t n, char *err, size_t errlen)
{
    if (n <= *cap)
        return 1;
    cudaFree(*buf);
    *buf = nullptr;
    *cap = 0;
    if (!tc_cu_check(cudaMalloc(buf, n * sizeof(SpState)), "cudaMalloc", err, errlen))
        return 0;
    *cap = n;
    return 1;
}

static int read_counters(unsigned long long *d_count, unsigned long long *d_nodes, int *d_found,
                         unsigned long long *count, unsigned long long *nodes, int *found,
                         char *err, size_t errlen)
{
    return tc_cu_check(cudaStreamSynchronize(tc_engine.stream), "super search", err, errlen) &&
           tc_cu_check(cudaMemcpy(count, d_count, 8, cudaMemcpyDeviceToHost), "copy", err,
                       errlen) &&
           tc_cu_check(cudaMemcpy(nodes, d_nodes, 8, cudaMemcpyDeviceToHost), "copy", err,
                       errlen) &&
           tc_cu_check(cudaMemcpy(found, d_found, sizeof(int), cudaMemcpyDeviceToHost), "copy",
                       err, errlen);
}

static int zero_counters(unsigned long long *d_count, unsigned long long *d_nodes, char *err,
                         size_t errlen)
{
    return tc_cu_check(cudaMemsetAsync(d_count, 0, 8, tc_engine.stream), "memset", err, errlen) &&
           tc_cu_check(cudaMemsetAsync(d_nodes, 0, 8, tc_engine.stream), "memset", err, errlen);
}

extern "C" int tc_super_run(const SpSpec *sp, int max_cost, int lb, int *found, int *cost,
                            int *below, SpState *sol, unsigned long long *nodes, double *seconds,
                            int quiet, char *err, size_t errlen)
{
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    double t0 = tc_now();
    *found = 0;
    *below = lb;
    *nodes = 0;
    SpSpec *d_spec = nullptr;
    int *d_found = nullptr;
    SpState *d_sol = nullptr;
    unsigned long long *d_next = nullptr, *d_nodes = nullptr, *d_count = nullptr;
    int ok = tc_cu_check(cudaMalloc(&d_spec, sizeof(SpSpec)), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMalloc(&d_found, sizeof(int)), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMalloc(&d_sol, sizeof(SpState)), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMalloc(&d_next, 8), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMalloc(&d_nodes, 8), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMalloc(&d_count, 8), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaMemcpy(d_spec, sp, sizeof(SpSpec), cudaMemcpyHostToDevice), "copy",
                         err, errlen);
    int per_sm = 0;
    if (ok)
        ok = tc_cu_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_super_kernel,
                                                                       128, 0),
                         "occupancy", err, errlen);
    const size_t threads = (size_t)tc_engine.sms * (per_sm > 0 ? per_sm : 1) * 128;
    SpState *lv[2] = {nullptr, nullptr};
    size_t lv_cap[2] = {0, 0};
    // the transposition table: 2^25 entries of 16 bytes, kept from budget to budget
    const unsigned long long tt_entries = 1ull << 25;
    ulonglong2 *d_tt = nullptr;
    ok = ok && tc_cu_check(cudaMalloc(&d_tt, tt_entries * sizeof(ulonglong2)), "cudaMalloc", err,
                           errlen) &&
         tc_cu_check(cudaMemset(d_tt, 0, tt_entries * sizeof(ulonglong2)), "memset", err, errlen);
    for (int budget = lb; ok && budget <= max_cost && !*found; budget++) {
        if (budget > DEV_LEVELS) {
            tc_fail(err, errlen, "budget %d is deeper than the device search goes (%d)", budget,
                    DEV_LEVELS);
            ok = 0;
            break;
        }
        // level 0, on the host: the root with every subset of the outputs RR already holds
        SpState root;
        sp_reset(sp, &root);
        int8_t list[SP_CELLS];
        const int k = sp_hits(sp, &root, list);
        SpState *top = (SpState *)tc_xmalloc(((size_t)1 << k) * sizeof(SpState));
        size_t n = 0;
        for (int mask = 0; mask < (1 << k) && !*found; mask++) {
            SpState x = root;
            sp_write(sp, &x, list, mask);
            (*nodes)++;
            const int a = sp_arrive(sp, &x, budget);
            if (a == 2) {
                *found = 1;
                *cost = x.cost;
                *sol = x;
            } else if (a == 0) {
                top[n++] = x;
            }
        }
        int cur = 0;
        if (!*found && n)
            ok = reserve(&lv[0], &lv_cap[0], n, err, errlen) &&
                 tc_cu_check(cudaMemcpy(lv[0], top, n * sizeof(SpState), cudaMemcpyHostToDevice),
                             "copy", err, errlen) &&
                 tc_cu_check(cudaMemset(d_found, 0, sizeof(int)), "memset", err, errlen);
        free(top);
        if (*found)
            n = 0;
        // the next levels, on the device, until one keeps every search thread busy
        for (int depth = 0; ok && n && n < FRONT_PER_THREAD * threads && depth < budget;) {
            SpExpand e = {d_spec, lv[cur], (unsigned long long)n, nullptr, d_count, d_nodes,
                          d_found, d_sol, budget};
            const unsigned blocks = (unsigned)((n + 127) / 128);
            unsigned long long kept = 0, dn = 0;
            int f = 0;
            ok = zero_counters(d_count, d_nodes, err, errlen);
            if (ok) {
                tc_super_expand<<<blocks, 128, 0, tc_engine.stream>>>(e);
                ok = tc_cu_check(cudaGetLastError(), "super expand", err, errlen) &&
                     read_counters(d_count, d_nodes, d_found, &kept, &dn, &f, err, errlen);
            }
            if (!ok)
                break;
            if (f) {
                *nodes += dn;
                *found = 1;
                ok = tc_cu_check(cudaMemcpy(sol, d_sol, sizeof(SpState), cudaMemcpyDeviceToHost),
                                 "copy", err, errlen);
                *cost = sol->cost;
                break;
            }
            if (kept > FRONT_MAX)  // too wide: search from this level (its children uncounted)
                break;
            *nodes += dn;
            if (!kept) {  // every child pruned: nothing at this budget
                n = 0;
                break;
            }
            ok = reserve(&lv[cur ^ 1], &lv_cap[cur ^ 1], kept, err, errlen) &&
                 tc_cu_check(cudaMemsetAsync(d_count, 0, 8, tc_engine.stream), "memset", err,
                             errlen);
            if (!ok)
                break;
            e.out = lv[cur ^ 1];
            tc_super_expand<<<blocks, 128, 0, tc_engine.stream>>>(e);
            ok = tc_cu_check(cudaGetLastError(), "super expand", err, errlen);
            cur ^= 1;
            n = (size_t)kept;
            depth++;
        }
        if (ok && !*found && n) {
            ok = tc_cu_check(cudaMemsetAsync(d_next, 0, 8, tc_engine.stream), "memset", err,
                             errlen) &&
                 tc_cu_check(cudaMemsetAsync(d_nodes, 0, 8, tc_engine.stream), "memset", err,
                             errlen);
            if (ok) {
                SpDev d = {d_spec, lv[cur], (unsigned long long)n, budget, d_next, d_found,
                           d_sol, d_nodes, d_tt, tt_entries - 1,
                           tc_super_tt_min_rem > 0 ? tc_super_tt_min_rem : 1};
                unsigned blocks = (unsigned)((n + 127) / 128);
                unsigned maxb = (unsigned)(tc_engine.sms * (per_sm > 0 ? per_sm : 1));
                if (blocks > maxb)
                    blocks = maxb;
                tc_super_kernel<<<blocks, 128, 0, tc_engine.stream>>>(d);
                ok = tc_cu_check(cudaGetLastError(), "super search", err, errlen) &&
                     tc_cu_check(cudaStreamSynchronize(tc_engine.stream), "super search", err,
                                 errlen);
            }
            int f = 0;
            unsigned long long dn = 0;
            ok = ok && tc_cu_check(cudaMemcpy(&f, d_found, sizeof f, cudaMemcpyDeviceToHost),
                                   "copy", err, errlen) &&
                 tc_cu_check(cudaMemcpy(&dn, d_nodes, 8, cudaMemcpyDeviceToHost), "copy", err,
                             errlen);
            *nodes += dn;
            if (ok && f) {
                ok = tc_cu_check(cudaMemcpy(sol, d_sol, sizeof(SpState), cudaMemcpyDeviceToHost),
                                 "copy", err, errlen);
                *found = 1;
                *cost = sol->cost;
            }
        }
        if (ok && !*found)
            *below = budget + 1;
        if (ok && !quiet)
            fprintf(stderr, "  cost %d: %s (%.3g nodes so far, %.1f s)\n", budget,
                    *found ? "found" : "none", (double)*nodes, tc_now() - t0);
    }
    cudaFree(lv[0]);
    cudaFree(lv[1]);
    cudaFree(d_tt);
    cudaFree(d_spec);
    cudaFree(d_found);
    cudaFree(d_sol);
    cudaFree(d_next);
    cudaFree(d_nodes);
    cudaFree(d_count);
    *seconds = tc_now() - t0;
    return ok;
}
