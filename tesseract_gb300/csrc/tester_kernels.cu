// Tester 1 on the device (the reference's t1_cycles, src/tester.c:94-168): every random program
// runs from 512 random states at once and Brent's algorithm finds the length of the cycle each
// run ends in.
//
// One block of 16 threads per program: thread j holds lanes 32j .. 32j + 31 (one 32-bit word of
// every cell).  The hare's cells and the tortoise's live in shared memory, cell c of thread j at
// [c * 16 + j]; RR in registers.  The instructions are the same for the whole block, so the
// loads of the code are broadcasts and every branch on them is uniform.
//
// Brent, as the reference runs it: the tortoise jumps to the hare at powers of two, the hare
// runs one pass at a time, and a lane's cycle length is the distance between them the first
// time the states are equal (RR and every writable cell).  The states are compared on a sample
// of up to 64 cells first, and in full only when some lane still searching passes the sample.
// At most max_passes passes: a lane without a cycle by then reports 0.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"
#include "tester.h"

#define T1_THREADS 16

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The n-th output (n >= 1) of splitmix64 started from s: its state has advanced n times.
__device__ __forceinline__ uint64_t splitmix_nth(uint64_t s, uint64_t n)
{
    return mix64(s + n * 0x9E3779B97F4A7C15ull);
}

__device__ __forceinline__ uint32_t run_pass(uint32_t *S, const uint32_t *code, uint32_t len,
                                             uint32_t r)
{
    uint32_t next = len ? __ldg(code) : 0u;
    for (uint32_t i = 0; i < len; i++) {
        const uint32_t in = next;
        if (i + 1 < len)
            next = __ldg(code + i + 1);
        uint32_t *cell = S + (in >> 1) * T1_THREADS;
        if (in & 1u)
            *cell = r;
        else
            r = ~(r & *cell);
    }
    return r;
}

__global__ void __launch_bounds__(T1_THREADS) tc_t1_kernel(TcT1Dev d)
{
    extern __shared__ uint32_t smem[];
    const uint32_t prog = blockIdx.x, j = threadIdx.x;
    const TcT1Job J = d.jobs[prog];
    const uint32_t ncells = J.ncells;
    uint32_t *H = smem + j, *Tt = smem + (size_t)ncells * T1_THREADS + j;
    const uint32_t *code = d.code + J.code;
    const uint32_t *sample = d.sample + J.sample;
    // t1_start (src/tester.c:84-91): cells 2.. then RR, eight 64-bit words each, from
    // splitmix64(seed ^ 0x5DEECE66D); this thread takes half j & 1 of word j >> 1
    const uint64_t s0 = J.seed ^ 0x5DEECE66Dull;
    const uint32_t w = j >> 1, half = (j & 1u) * 32u;
    H[0] = 0u;
    H[T1_THREADS] = 0xffffffffu;
    for (uint32_t c = 2; c < ncells; c++)
        H[c * T1_THREADS] = (uint32_t)(splitmix_nth(s0, (uint64_t)(c - 2) * 8 + w + 1) >> half);
    uint32_t r = (uint32_t)(splitmix_nth(s0, (uint64_t)(ncells - 2) * 8 + w + 1) >> half);
    // the tortoise starts where the hare does; the hare takes one pass
    for (uint32_t c = 0; c < ncells; c++)
        Tt[c * T1_THREADS] = H[c * T1_THREADS];
    uint32_t rt = r;
    r = run_pass(H, code, J.len, r);
    uint64_t lam = 1, power = 1, steps = 1;
    uint32_t active = 0xffffffffu;
    uint64_t *lam_out = d.lam + (size_t)prog * 512 + 32 * j;
    for (uint32_t l = 0; l < 32; l++)
        lam_out[l] = 0;
    const unsigned group = 0xffffu;  // the block's 16 threads: lanes 0..15 of its warp
    for (;;) {
        uint32_t diff = r ^ rt;
        for (uint32_t i = 0; i < J.nsample; i++)
            diff |= H[sample[i] * T1_THREADS] ^ Tt[sample[i] * T1_THREADS];
        if (J.nsample < ncells - 2 && __any_sync(group, (active & ~diff) != 0u)) {
            diff = r ^ rt;
            for (uint32_t c = 2; c < ncells; c++)
                diff |= H[c * T1_THREADS] ^ Tt[c * T1_THREADS];
        }
        for (uint32_t found = active & ~diff; found; found &= found - 1u)
            lam_out[__ffs(found) - 1] = lam;
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
        r = run_pass(H, code, J.len, r);
        lam++;
        steps++;
    }
    if (j == 0)
        d.passes[prog] = steps;
}

extern "C" int tc_t1_launch(const TcT1Dev *d, uint32_t nprogs, uint32_t max_cells,
                            cudaStream_t stream, char *err, size_t errlen)
{
    const size_t smem = (size_t)2 * max_cells * T1_THREADS * sizeof(uint32_t);
    if (smem > (size_t)tc_engine.smem_optin)
        return tc_fail(err, errlen, "tester1 on the GPU holds at most %zu cells per machine",
                       (size_t)tc_engine.smem_optin / (2 * T1_THREADS * sizeof(uint32_t)) - 2);
    if (!tc_cu_check(cudaFuncSetAttribute(tc_t1_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem),
                     "tester1 smem", err, errlen))
        return 0;
    tc_t1_kernel<<<nprogs, T1_THREADS, smem, stream>>>(*d);
    return tc_cu_check(cudaGetLastError(), "tester1 launch", err, errlen);
}
