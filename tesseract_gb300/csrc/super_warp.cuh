// The superoptimizer's device search: one warp per frontier subtree (included by
// super_kernels.cu).
#ifndef TC_SUPER_WARP_CUH
#define TC_SUPER_WARP_CUH

#include "super_search.cuh"

#ifndef DEV_LEVELS
#define DEV_LEVELS 44      // deepest level a device search reaches (budgets up to 44)
#endif
#define POLL 1024          // nodes between looks at the stop flag

// ---- device: depth-first search of one subtree per warp -----------------------------------------
//
// A warp searches one frontier subtree at a time, its 32 lanes on the same node: the search's
// control flow is the same in every lane, and the work of a node (the operands a NAND may read,
// one per value, the cheapest; the transposition-table keys; the lower bound; the outputs the new
// RR value can write) is spread over the lanes with ballots and match_any.  One search per
// thread, the reference's layout, diverges at every branch of the search and keeps ~3.6 KB of
// state per thread in local memory; here the state is a few registers, equal in every lane, and
// the warp's stack of levels in shared memory.
//
// Operands are numbered compactly: 0 ZERO, 1 ONE, 2 + c cell c, 2 + ncells + j the RR value
// hist[j]; lane l evaluates operands l and l + 32.  This is the reference's order (ZERO, ONE, the
// cells, then RR values; src/super.c:373-406), so children are visited in the same order.

#define FULL 0xffffffffu
#define LV (DEV_LEVELS + 1)
#define SUB_DONE 0x80000000u  // every subset of a level's outputs has been tried

struct SpDev {
    const SpSpec *spec;
    const SpState *frontier;
    unsigned long long nfront;
    int budget;
    unsigned long long *next;
    int *found;
    SpState *sol;
    unsigned long long *nodes;
    ulonglong2 *tt;             // the transposition table, shared by every warp
    unsigned long long tt_mask;
    int tt_min_rem;             // states with fewer instructions left are not looked up
};


// One warp's levels: what the DFS takes back on the way up.
struct WarpStack {
    uint64_t hist[LV];           // RR after NAND j
    uint64_t keep[LV];           // the operands of level L's node, one per value
    uint64_t key1[LV], key2[LV];
    uint32_t w_readable[LV], w_written[LV], used_before[LV];
    uint32_t hits[LV], sub[LV];  // the outputs NAND L can write; the subset being tried
    int16_t  w_cost[LV];
    uint8_t  ci[LV], opk[LV];
    int8_t   opr[LV], key_rem[LV];
};

// The node the warp is at; every lane holds the same values.
struct WNode {
    uint64_t rr, stored;         // hist[n]; bit j: hist[j] has been stored
    uint32_t readable, written, used;
    int      n, cost, def0;
};

// What a lane knows of the spec: as operand `lane` (a cell for 2 <= lane < 2 + ncells) and as
// cell `lane` (for the outputs).
struct LaneSpec {
    uint64_t op_init, op_target, target;
    int      op_sym;
    bool     op_cell, out;
};

// This lane's two operands.
struct Ops {
    uint64_t vA, vB;
    bool     okA, okB, e0A, e0B;  // e0: costs no store
};

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The operands a NAND may read at node x, one per value: the cheapest, and the first of those
// (sp_build's rule).  Returns them as a bit set over operand numbers.
__device__ uint64_t warp_survivors(const SpSpec *sp, const WarpStack &ws, const WNode &x,
                                   const LaneSpec &ls, int base, Ops &o)
{
    const int lane = threadIdx.x & 31;
    if (lane == 0) {
        o.okA = true; o.vA = 0; o.e0A = true;
    } else if (lane == 1) {
        o.okA = true; o.vA = sp->mask; o.e0A = true;
    } else if (ls.op_cell) {
        const int c = lane - 2;
        o.okA = ((x.readable >> c) & 1) && (ls.op_sym < 0 || ((x.used >> ls.op_sym) & 1));
        o.vA = ((x.written >> c) & 1) ? ls.op_target : ls.op_init;
        o.e0A = true;
    } else {
        const int j = lane - base;
        o.okA = j <= x.n && (j > 0 || x.def0);
        o.vA = o.okA ? ws.hist[j] : 0;
        o.e0A = o.okA && ((x.stored >> j) & 1);
    }
    const int jB = lane + 32 - base;  // >= 14: an RR value
    o.okB = jB <= x.n;
    o.vB = o.okB ? ws.hist[jB] : 0;
    o.e0B = o.okB && ((x.stored >> jB) & 1);
    const uint32_t okA = __ballot_sync(FULL, o.okA), zeroA = __ballot_sync(FULL, o.okA && o.e0A);
    bool winA = false;
    if (o.okA) {
        const uint32_t m = __match_any_sync(okA, o.vA), z = m & zeroA;
        winA = __ffs(z ? z : m) - 1 == lane;
    }
    uint32_t keepA = __ballot_sync(FULL, winA), keepB = 0;
    const uint32_t okB = __ballot_sync(FULL, o.okB);
    if (okB) {
        const uint32_t zeroB = __ballot_sync(FULL, o.okB && o.e0B);
        uint32_t classB = 0;
        bool winB = false;
        if (o.okB) {
            classB = __match_any_sync(okB, o.vB);
            const uint32_t z = classB & zeroB;
            winB = __ffs(z ? z : classB) - 1 == lane;
        }
        keepB = __ballot_sync(FULL, winB);
        // a value held by operands of both halves: the A side has the lower numbers
        for (uint32_t rest = keepB; rest; rest &= rest - 1) {
            const int src = __ffs(rest) - 1;
            const uint64_t v = __shfl_sync(FULL, o.vB, src);
            const uint32_t cls = __shfl_sync(FULL, classB, src);
            const uint32_t eqA = __ballot_sync(FULL, o.okA && o.vA == v);
            if (!eqA)
                continue;
            if (!(eqA & zeroA) && (cls & zeroB))
                keepA &= ~eqA;             // only the B side has a free one
            else
                keepB &= ~(1u << src);
        }
    }
    return (uint64_t)keepB << 32 | keepA;
}

// The transposition-table keys of node x (the reference's, src/super.c:626-641): RR, the cell
// masks, and the operand values with their costs as a set (a sum over the lanes).
__device__ void warp_key(const WNode &x, uint64_t keep, const Ops &o, uint64_t *k1,
                         uint64_t *k2)
{
    const int lane = threadIdx.x & 31;
    uint64_t a = mix64(x.rr ^ (uint64_t)(x.n > 0 || x.def0) << 63), b = mix64(a + 0x1234567);
    const uint64_t f = (uint64_t)x.readable | (uint64_t)x.written << 21 | (uint64_t)x.used << 42;
    a += mix64(f + 0x9E3779B97F4A7C15ull);
    b ^= mix64(f * 3 + 77);
    // an operand that costs a store is told apart by a constant XORed in (not by a shift, which
    // would lose the top row of a 64-row table)
    const uint64_t lazy = 0xD6E8FEB86659FD93ull;
    uint64_t ca = 0, cb = 0;
    if ((keep >> lane) & 1) {
        const uint64_t v = o.vA ^ (o.e0A ? 0ull : lazy);
        ca += mix64(v + 0x51ED27);
        cb += mix64(v * 0x2545F4914F6CDD1Dull + 0xABCDEF);
    }
    if ((keep >> (lane + 32)) & 1) {
        const uint64_t v = o.vB ^ (o.e0B ? 0ull : lazy);
        ca += mix64(v + 0x51ED27);
        cb += mix64(v * 0x2545F4914F6CDD1Dull + 0xABCDEF);
    }
    const uint32_t alo = __reduce_add_sync(FULL, (uint32_t)ca);
    const uint32_t ahi = __reduce_add_sync(FULL, (uint32_t)(ca >> 32));
    const uint32_t blo = __reduce_add_sync(FULL, (uint32_t)cb);
    const uint32_t bhi = __reduce_add_sync(FULL, (uint32_t)(cb >> 32));
    *k1 = a + ((uint64_t)ahi << 32 | alo);
    *k2 = b + ((uint64_t)bhi << 32 | blo);
}

// sp_arrive for the warp: 0 go on, 1 pruned, 2 goal.  The lower bound (sp_lower_bound): one STO
// per unwritten output, one NAND per distinct target among them that RR does not hold, and RR's
// own target.
__device__ int warp_arrive(const SpSpec *sp, const WNode &x, const LaneSpec &ls,
                           uint32_t out_mask, int budget)
{
    if (x.cost > budget)
        return 1;
    const bool def = x.n > 0 || x.def0;
    const uint32_t U = out_mask & ~x.written;
    if (!U && (!sp->rr_out || (def && x.rr == sp->rr_target)))
        return 2;
    const int lane = threadIdx.x & 31;
    const bool mine = (U >> lane) & 1, held = def && ls.target == x.rr;
    bool lead = false;
    if (mine) {
        const uint32_t m = __match_any_sync(U, ls.target);
        lead = __ffs(m) - 1 == lane;
    }
    const uint32_t need = __ballot_sync(FULL, mine && lead && !held);
    int nands = __popc(need);
    if (sp->rr_out) {
        const bool in_need =
            __ballot_sync(FULL, mine && !held && ls.target == sp->rr_target) != 0;
        if (!(def && x.rr == sp->rr_target)) {
            if (!in_need)
                nands++;
        } else if (need) {
            nands++;
        }
    }
    if (x.cost + __popc(U) + nands > budget || x.n == SP_LEN)
        return 1;
    return 0;
}

// The operands whose NAND leads to a child worth visiting: sp_nand's checks (RR defined or the
// operand ZERO; RR changes) and the child's lower bound.  The bound is the same for every subset
// of the outputs the child then writes (each write adds one instruction and takes one STO off
// the bound; the outputs it writes hold RR's value, which the bound leaves out already), and a
// child over the bound can be no goal, so such children are dropped here, in one pass over all
// operands, instead of one visit each.
__device__ uint64_t warp_filter(const SpSpec *sp, const WNode &x, uint64_t keep, const Ops &o,
                                const LaneSpec &ls, uint32_t out_mask, int budget, int L)
{
    if (L + 1 > DEV_LEVELS)
        return 0;
    const int lane = threadIdx.x & 31;
    const bool def = x.n > 0 || x.def0;
    if (!def)
        keep &= 1ull;  // only ZERO may be read before RR is defined
    const uint32_t U = out_mask & ~x.written;
    // distinct targets among the unwritten outputs
    bool lead = false;
    if ((U >> lane) & 1) {
        const uint32_t m = __match_any_sync(U, ls.target);
        lead = __ffs(m) - 1 == lane;
    }
    const int distinct = __popc(__ballot_sync(FULL, lead));
    bool rrt_in_u = false;
    uint64_t r[2];
    bool in_u[2] = {false, false};
    r[0] = ~(x.rr & o.vA) & sp->mask;
    r[1] = ~(x.rr & o.vB) & sp->mask;
    for (uint32_t u = U; u; u &= u - 1) {
        const uint64_t t = sp->target[__ffs(u) - 1];
        in_u[0] |= t == r[0];
        in_u[1] |= t == r[1];
        rrt_in_u |= t == sp->rr_target;
    }
    const int base_cost = x.cost + 1 + __popc(U);
    bool pass[2];
    for (int h = 0; h < 2; h++) {
        const int need = distinct - in_u[h];
        int nands = need;
        if (sp->rr_out) {
            if (r[h] != sp->rr_target) {
                if (!(rrt_in_u && sp->rr_target != r[h]))
                    nands++;
            } else if (need) {
                nands++;
            }
        }
        const int extra = h == 0 ? !o.e0A : !o.e0B;
        pass[h] = !(def && r[h] == x.rr) && base_cost + extra + nands <= budget;
    }
    const uint64_t ok = (uint64_t)__ballot_sync(FULL, pass[0]) |
                        (uint64_t)__ballot_sync(FULL, pass[1]) << 32;
    return keep & ok;
}

// ---- the transposition table ------------------------------------------------------------------
//
// States searched in full without a program, as the reference's per-thread table keeps them
// (src/super.c:408-418, 641-716): the same state is reached in many orders, and its future
// depends only on RR, the readable, written and used cells, and the values a NAND could read with
// what each costs.  Here one table serves every warp, and it is kept from budget to budget.  An
// entry is two 64-bit words: the state's first key, and its second key with the low byte
// replaced by the instructions that were left when it was searched; a state arriving with `rem`
// left is pruned when an entry holds both its keys and at least `rem`.  An entry torn between two
// writers matches only when both wrote this state (the rem is then a true one) or by a 120-bit
// coincidence, which the reference's 128-bit keys also rule out in practice.

// Other warps write the table and the found flag while this one runs, so lane 0 reads them and
// the warp takes its answer: lanes that read for themselves could see different values and part
// ways.
__device__ __forceinline__ bool tt_seen(const SpDev &d, uint64_t k1, uint64_t k2, int rem)
{
    int seen = 0;
    if ((threadIdx.x & 31) == 0) {
        const ulonglong2 e = d.tt[k1 & d.tt_mask];
        seen = e.x == k1 && (e.y & ~0xFFull) == (k2 & ~0xFFull) && (int)(e.y & 0xFFull) >= rem;
    }
    return __shfl_sync(FULL, seen, 0) != 0;
}

__device__ __forceinline__ bool found_flag(const SpDev &d)
{
    int f = 0;
    if ((threadIdx.x & 31) == 0)
        f = *(volatile int *)d.found;
    return __shfl_sync(FULL, f, 0) != 0;
}

__device__ __forceinline__ void tt_store(const SpDev &d, uint64_t k1, uint64_t k2, int rem)
{
    d.tt[k1 & d.tt_mask] = make_ulonglong2(k1, (k2 & ~0xFFull) | (uint64_t)rem);
}

// The warp's lanes all read and write the stack with the same values; a __syncwarp between a
// read and the write that replaces it keeps a lane that runs ahead from changing what another
// lane has yet to read.
__device__ __forceinline__ void next_subset(WarpStack &ws, int L)
{
    const uint32_t s = ws.sub[L], h = ws.hits[L];
    __syncwarp();
    ws.sub[L] = s == h ? SUB_DONE : (s - h) & h;  // the subsets of h in increasing order
}

#define WARPS 4

__global__ void __launch_bounds__(WARPS * 32) tc_super_kernel(SpDev d)
{
    __shared__ SpSpec sp_s;
    __shared__ WarpStack stacks[WARPS];
    if (threadIdx.x == 0)
        sp_s = *d.spec;
    __syncthreads();
    const SpSpec *sp = &sp_s;
    const int lane = threadIdx.x & 31;
    WarpStack &ws = stacks[threadIdx.x >> 5];
    const int base = 2 + sp->ncells;
    LaneSpec ls;
    ls.op_cell = lane >= 2 && lane < base;
    ls.op_init = ls.op_cell ? sp->init[lane - 2] : 0;
    ls.op_target = ls.op_cell ? sp->target[lane - 2] : 0;
    ls.op_sym = ls.op_cell ? sp->sym_prev[lane - 2] : -1;
    ls.out = lane < sp->ncells && sp->out[lane];
    ls.target = lane < sp->ncells ? sp->target[lane] : 0;
    const uint32_t out_mask = __ballot_sync(FULL, ls.out);
    unsigned long long nodes = 0, polled = 0;
    const int budget = d.budget;
    for (;;) {
        unsigned long long f = 0;
        if (lane == 0)
            f = atomicAdd(d.next, 1ull);
        f = __shfl_sync(FULL, f, 0);
        if (f >= d.nfront || found_flag(d))
            break;
        const SpState *src = d.frontier + f;
        WNode x;
        x.n = src->n;
        x.cost = src->cost;
        x.readable = src->readable;
        x.written = src->written;
        x.used = src->used;
        x.def0 = src->def0;
        for (int j = lane; j <= x.n; j += 32) {
            ws.hist[j] = src->hist[j];
            ws.opk[j] = src->op_kind[j];
            ws.opr[j] = src->op_ref[j];
        }
        x.stored = (uint64_t)__ballot_sync(FULL, lane <= x.n && src->stored[lane]) |
                   (uint64_t)__ballot_sync(FULL, lane + 32 <= x.n && src->stored[lane + 32])
                       << 32;
        int out_at = lane < SP_CELLS ? src->out_at[lane] : -1;  // cell `lane`
        __syncwarp();
        x.rr = ws.hist[x.n];
        const int n0 = x.n;
        int L = n0;
        Ops o;
        ws.keep[L] = warp_filter(sp, x, warp_survivors(sp, ws, x, ls, base, o), o, ls, out_mask,
                                 budget, L);
        ws.ci[L] = 0;
        ws.key_rem[L] = -1;
        bool expand = true, stop = false;
        for (;;) {
            __syncwarp();
            if (nodes - polled >= POLL) {
                polled = nodes;
                if (found_flag(d))
                    break;
            }
            if (expand) {
                const uint64_t rest = ws.keep[L] & (~0ull << ws.ci[L]);
                if (!rest) {  // every operand tried at this level
                    if (L == n0)
                        break;
                    if (ws.key_rem[L] >= 0 && lane == 0)  // searched in full, nothing found
                        tt_store(d, ws.key1[L], ws.key2[L], ws.key_rem[L]);
                    x.readable = ws.w_readable[L];
                    x.written = ws.w_written[L];
                    x.cost = ws.w_cost[L];
                    next_subset(ws, L);
                    expand = false;
                    continue;
                }
                const int i = __ffsll((long long)rest) - 1;
                __syncwarp();
                ws.ci[L] = (uint8_t)(i + 1);
                uint64_t v;
                int kind, ref = 0, extra = 0;
                if (i == 0) {
                    v = 0;
                    kind = SK_ZERO;
                } else if (i == 1) {
                    v = sp->mask;
                    kind = SK_ONE;
                } else if (i < base) {
                    ref = i - 2;
                    v = ((x.written >> ref) & 1) ? sp->target[ref] : sp->init[ref];
                    kind = SK_CELL;
                } else {
                    ref = i - base;
                    v = ws.hist[ref];
                    kind = ((x.stored >> ref) & 1) ? SK_TEMP : SK_LAZY;
                    extra = kind == SK_LAZY;
                }
                // sp_nand's checks
                const bool def = x.n > 0 || x.def0;
                const uint64_t r = ~(x.rr & v) & sp->mask;
                if ((!def && kind != SK_ZERO) || (def && r == x.rr) ||
                    x.cost + 1 + extra > budget || L + 1 > DEV_LEVELS)
                    continue;
                if (kind == SK_LAZY)
                    x.stored |= 1ull << ref;
                const uint32_t used = x.used;
                if (kind == SK_CELL)
                    x.used |= 1u << ref;
                x.cost += 1 + extra;
                x.n++;
                L++;
                x.rr = r;
                ws.hist[L] = r;
                ws.opk[L] = (uint8_t)kind;
                ws.opr[L] = (int8_t)ref;
                ws.used_before[L] = used;
                ws.hits[L] = __ballot_sync(FULL, ls.out && !((x.written >> lane) & 1) &&
                                                     ls.target == r);
                ws.sub[L] = 0;
                expand = false;
                continue;
            }
            // the output writes after NAND L
            const uint32_t S = ws.sub[L];
            if (S & SUB_DONE) {  // all tried: take the NAND back
                const bool lazy = ws.opk[L] == SK_LAZY;
                if (lazy)
                    x.stored &= ~(1ull << ws.opr[L]);
                x.cost -= 1 + lazy;
                x.used = ws.used_before[L];
                x.n--;
                L--;
                x.rr = ws.hist[L];
                expand = true;
                continue;
            }
            ws.w_readable[L] = x.readable;
            ws.w_written[L] = x.written;
            ws.w_cost[L] = (int16_t)x.cost;
            for (uint32_t s = S; s; s &= s - 1) {  // sp_write
                const int c = __ffs(s) - 1;
                x.written |= 1u << c;
                x.cost++;
                x.readable &= ~sp->alias[c];
                x.readable |= 1u << c;
            }
            if ((S >> lane) & 1)
                out_at = x.n;
            nodes++;
            const int a = warp_arrive(sp, x, ls, out_mask, budget);
            if (a == 2) {
                int won = 0;
                if (lane == 0)
                    won = atomicCAS(d.found, 0, 1) == 0;
                if (__shfl_sync(FULL, won, 0)) {
                    SpState *sol = d.sol;
                    if (lane == 0) {
                        sol->n = x.n;
                        sol->cost = x.cost;
                        sol->readable = x.readable;
                        sol->written = x.written;
                        sol->used = x.used;
                        sol->def0 = x.def0;
                    }
                    for (int j = lane; j <= x.n; j += 32) {
                        sol->hist[j] = ws.hist[j];
                        sol->stored[j] = (uint8_t)((x.stored >> j) & 1);
                        sol->op_kind[j] = ws.opk[j];
                        sol->op_ref[j] = ws.opr[j];
                    }
                    if (lane < SP_CELLS)
                        sol->out_at[lane] = (int8_t)out_at;
                }
                stop = true;
                break;
            }
            if (a == 0) {
                const uint64_t all = warp_survivors(sp, ws, x, ls, base, o);
                ws.keep[L] = warp_filter(sp, x, all, o, ls, out_mask, budget, L);
                ws.ci[L] = 0;
                ws.key_rem[L] = -1;
                const int rem = budget - x.cost;
                bool seen = false;
                if (rem >= d.tt_min_rem) {  // small subtrees: cheaper to search again
                    uint64_t k1, k2;
                    warp_key(x, all, o, &k1, &k2);
                    ws.key1[L] = k1;
                    ws.key2[L] = k2;
                    seen = tt_seen(d, k1, k2, rem);
                    ws.key_rem[L] = (int8_t)rem;
                }
                if (!seen) {
                    expand = true;
                    continue;
                }
                ws.key_rem[L] = -1;  // searched before with at least this much left: nothing there
            }
            x.readable = ws.w_readable[L];
            x.written = ws.w_written[L];
            x.cost = ws.w_cost[L];
            next_subset(ws, L);
        }
        if (stop || found_flag(d))
            break;
    }
    if (lane == 0)
        atomicAdd(d.nodes, nodes);
}

#endif
