// The superoptimizer on the GPU: iterative deepening over the budget.  For each budget the top of
// the search tree is expanded breadth-first on the device, one kernel per level, until the level
// holds enough states to keep every warp busy; then every warp runs an explicit-stack depth-first
// search of frontier subtrees taken from a work queue.  The search model and its
// pruning are in super_search.cuh; the first thread to reach the goal records its state and
// raises a flag the others poll, as the reference's threads share one stop flag
// (src/super.c:770-896).
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "engine.h"
#include "super_search.cuh"
#include "super_warp.cuh"

#define FRONT_PER_WARP 64    // frontier states per searching warp, for the work queue's balance
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

// Subtrees with fewer instructions left than this are searched again rather than looked up:
// a lookup is a random global-memory access.
extern "C" {
int tc_super_tt_min_rem = 4;
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
                                                                       WARPS * 32, 0),
                         "occupancy", err, errlen);
    const size_t warps = (size_t)tc_engine.sms * (per_sm > 0 ? per_sm : 1) * WARPS;
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
        for (int depth = 0; ok && n && n < FRONT_PER_WARP * warps && depth < budget;) {
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
                unsigned blocks = (unsigned)((n + WARPS - 1) / WARPS);
                unsigned maxb = (unsigned)(tc_engine.sms * (per_sm > 0 ? per_sm : 1));
                if (blocks > maxb)
                    blocks = maxb;
                tc_super_kernel<<<blocks, WARPS * 32, 0, tc_engine.stream>>>(d);
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
