// Tester 1 on the device (the reference's t1_cycles, src/tester.c:94-168, with t1_work's
// bookkeeping, src/tester.c:182-223): every random program runs from 512 random states at once
// and Brent's algorithm finds the length of the cycle each run ends in.
//
// One block of 16 threads per program: thread j holds lanes 32j .. 32j + 31 (one 32-bit word of
// every cell).  The block first writes its program into shared memory: instruction i comes from
// output i + 1 of splitmix64 started at the program's seed, and the n-th output of splitmix64 is
// a function of n, so the 16 threads make the instructions side by side (random_program,
// src/tester.c:57-81; the seed is t1_program_seed, src/tester.c:51-55).  The hare's cells and the
// tortoise's live in shared memory too, cell c of thread j at [c * 16 + j]; RR in registers.  The
// instructions are the same for the whole block, so every branch on them is uniform.
//
// Brent, as the reference runs it: the tortoise jumps to the hare at powers of two, the hare
// runs one pass at a time, and a lane's cycle length is the distance between them the first
// time the states are equal (RR and every writable cell).  The states are compared on a sample
// of up to 64 cells first, and in full only when some lane still searching passes the sample.
// At most max_passes passes: a lane without a cycle by then counts as "none".
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"
#include "tester.h"

#define T1_THREADS 16
#define GOLDEN 0x9E3779B97F4A7C15ull

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Output n (n >= 1) of splitmix64 started from state s.
__device__ __forceinline__ uint64_t splitmix_nth(uint64_t s, uint64_t n)
{
    return mix64(s + n * GOLDEN);
}

__device__ __forceinline__ uint32_t run_one(uint32_t *S, uint32_t in, uint32_t r)
{
    uint32_t *cell = S + (in >> 1) * T1_THREADS;
    if (in & 1u)
        *cell = r;
    else
        r = ~(r & *cell);
    return r;
}

// One pass; the instructions are read four at a time (one 16-byte shared-memory load; the code
// starts the block's dynamic shared memory, so it is 16-byte aligned).
__device__ __forceinline__ uint32_t run_pass(uint32_t *S, const uint32_t *code, uint32_t len,
                                             uint32_t r)
{
    const uint4 *code4 = (const uint4 *)code;
    uint32_t i = 0;
    for (; i + 4 <= len; i += 4) {
        const uint4 q = code4[i >> 2];
        r = run_one(S, q.x, r);
        r = run_one(S, q.y, r);
        r = run_one(S, q.z, r);
        r = run_one(S, q.w, r);
    }
    for (; i < len; i++)
        r = run_one(S, code[i], r);
    return r;
}

__device__ __forceinline__ int bucket(uint64_t lam)
{
    int b = 0;
    while (b < T1_BUCKETS - 2 && (1ull << b) < lam)
        b++;
    return b;
}

__global__ void __launch_bounds__(T1_THREADS) tc_t1_kernel(TcT1Dev d)
{
    extern __shared__ __align__(16) uint32_t smem[];
    __shared__ unsigned long long hist[T1_BUCKETS];
    const uint32_t j = threadIdx.x;
    const uint64_t k = d.k0 + blockIdx.x;
    const uint32_t cells = d.cells, ncells = cells + 2u, len = d.len;
    uint32_t *code = smem;
    uint32_t *H = smem + len + j, *Tt = smem + len + (size_t)ncells * T1_THREADS + j;
    // t1_program_seed: splitmix64 once from seed ^ cells << 40 ^ k * 0xD1B54A32D192ED03
    const uint64_t ps = splitmix_nth(d.seed ^ ((uint64_t)cells << 40) ^
                                         (k * 0xD1B54A32D192ED03ull), 1);
    for (uint32_t i = j; i < len; i += T1_THREADS) {
        const uint64_t r = splitmix_nth(ps, (uint64_t)i + 1);
        const uint32_t op = (uint32_t)(r & 1u);
        const uint32_t addr = op == 0u ? (uint32_t)((r >> 1) % ncells)
                                       : 2u + (uint32_t)((r >> 1) % cells);
        code[i] = addr << 1 | op;
    }
    for (uint32_t b = j; b < T1_BUCKETS; b += T1_THREADS)
        hist[b] = 0;
    // t1_start (src/tester.c:84-91): cells 2.. then RR, eight 64-bit words each, from
    // splitmix64(seed ^ 0x5DEECE66D); this thread takes half j & 1 of word j >> 1
    const uint64_t s0 = ps ^ 0x5DEECE66Dull;
    const uint32_t w = j >> 1, half = (j & 1u) * 32u;
    H[0] = 0u;
    H[T1_THREADS] = 0xffffffffu;
    for (uint32_t c = 2; c < ncells; c++)
        H[c * T1_THREADS] = (uint32_t)(splitmix_nth(s0, (uint64_t)(c - 2) * 8 + w + 1) >> half);
    uint32_t r = (uint32_t)(splitmix_nth(s0, (uint64_t)cells * 8 + w + 1) >> half);
    for (uint32_t c = 0; c < ncells; c++)
        Tt[c * T1_THREADS] = H[c * T1_THREADS];
    __syncwarp(0xffffu);  // the code and the histogram are shared by the block's one warp
    uint32_t rt = r;
    r = run_pass(H, code, len, r);
    uint64_t lam = 1, power = 1, steps = 1, longest = 0;
    uint32_t active = 0xffffffffu;
    const unsigned group = 0xffffu;  // the block's 16 threads: lanes 0..15 of its warp
    for (;;) {
        uint32_t diff = r ^ rt;
        for (uint32_t i = 0; i < d.nsample; i++) {
            const uint32_t c = 2u + (uint32_t)((uint64_t)i * cells / d.nsample);
            diff |= H[c * T1_THREADS] ^ Tt[c * T1_THREADS];
        }
        if (d.nsample < cells && __any_sync(group, (active & ~diff) != 0u)) {
            diff = r ^ rt;
            for (uint32_t c = 2; c < ncells; c++)
                diff |= H[c * T1_THREADS] ^ Tt[c * T1_THREADS];
        }
        const uint32_t found = active & ~diff;
        if (found) {
            atomicAdd(&hist[bucket(lam)], (unsigned long long)__popc(found));
            longest = lam > longest ? lam : longest;
        }
        active &= diff;
        if (!__any_sync(group, active != 0u) || steps >= d.max_passes)
            break;
        if (power == lam) {
            for (uint32_t c = 2; c < ncells; c++)
                Tt[c * T1_THREADS] = H[c * T1_THREADS];
            rt = r;
            power *= 2;
            lam = 0;
        }
        r = run_pass(H, code, len, r);
        lam++;
        steps++;
    }
    if (active)
        atomicAdd(&hist[T1_BUCKETS - 1], (unsigned long long)__popc(active));
    for (int o = 8; o > 0; o >>= 1) {
        const uint64_t other = __shfl_xor_sync(group, longest, o);
        longest = other > longest ? other : longest;
    }
    __syncwarp(0xffffu);
    for (uint32_t b = j; b < T1_BUCKETS; b += T1_THREADS)
        if (hist[b])
            atomicAdd((unsigned long long *)d.hist + b, hist[b]);
    if (j == 0) {
        d.passes[blockIdx.x] = steps;
        d.longest[blockIdx.x] = longest;
    }
}

extern "C" int tc_t1_launch(const TcT1Dev *d, uint32_t nprogs, cudaStream_t stream, char *err,
                            size_t errlen)
{
    const size_t smem = ((size_t)d->len + (size_t)2 * (d->cells + 2) * T1_THREADS) *
                        sizeof(uint32_t);
    if (smem > (size_t)tc_engine.smem_optin)
        return tc_fail(err, errlen, "tester1 on the GPU holds a %u-cell machine of %u "
                       "instructions in %zu bytes of shared memory; this one needs %zu",
                       d->cells, d->len, (size_t)tc_engine.smem_optin, smem);
    if (!tc_cu_check(cudaFuncSetAttribute(tc_t1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem),
                     "tester1 smem", err, errlen))
        return 0;
    tc_t1_kernel<<<nprogs, T1_THREADS, smem, stream>>>(*d);
    return tc_cu_check(cudaGetLastError(), "tester1 launch", err, errlen);
}
