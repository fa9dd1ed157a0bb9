// The batched engine's device side: one persistent kernel runs thousands of enumeration jobs of
// uneven length, cell count and input width from a device work queue.
//
// A work unit is J.unit_words consecutive 32-lane words of one job (TC_BATCH_UNIT_WORDS, or fewer
// in a wave too small to fill the GPU with units of that size).  Each block takes
// units from a global counter until none are left; each thread runs one word at a time.  The
// programs are interpreted from their packed bundles (batch.h) with every cell in shared memory
// (one 32-bit word per thread and slot, bank-conflict free), RR in a register.  The bundle words
// are the same for the whole block, so their loads are broadcasts.
//
// Results: hits per job (one atomic per unit), and per unit the first 16 hits in assignment
// order, which the host merges into each job's 16 smallest.
#include <cuda_runtime.h>
#include <stdint.h>

#include "batch.h"
#include "engine.h"

#define B TC_BATCH_BLOCK


__device__ __forceinline__ uint32_t lane_word(uint64_t w, int j)
{
    const uint32_t pat[5] = {0xaaaaaaaau, 0xccccccccu, 0xf0f0f0f0u, 0xff00ff00u, 0xffff0000u};
    return j < 5 ? pat[j] : 0u - (uint32_t)((w >> (j - 5)) & 1ull);
}

// One pass of a packed program over this thread's word: S points at the thread's column.
__device__ __forceinline__ uint32_t run_program(uint32_t *S, const uint64_t *code, uint32_t nb,
                                                uint32_t r)
{
    uint64_t next = nb ? __ldg(code) : 0;
    for (uint32_t i = 0; i < nb; i++) {
        const uint64_t b = next;
        if (i + 1 < nb)
            next = __ldg(code + i + 1);
        const uint32_t lo = (uint32_t)b, hi = (uint32_t)(b >> 32);
        const uint32_t nN = lo & 15u, nS = (lo >> 4) & 15u;
        const uint32_t x0 = S[((lo >> 8) & 255u) * B];
        const uint32_t x1 = S[((lo >> 16) & 255u) * B];
        const uint32_t x2 = S[(lo >> 24) * B];
        const uint32_t x3 = S[(hi & 255u) * B];
        if (nN > 0u) r = ~(r & x0);
        if (nN > 1u) r = ~(r & x1);
        if (nN > 2u) r = ~(r & x2);
        if (nN > 3u) r = ~(r & x3);
        if (nS > 0u) S[((hi >> 8) & 255u) * B] = r;
        if (nS > 1u) S[((hi >> 16) & 255u) * B] = r;
        if (nS > 2u) S[(hi >> 24) * B] = r;
    }
    return r;
}

// A 3-input LUT with a truth table known only at run time: the table is the same for the whole
// block, so a jump on it is uniform and each case is one lop3.b32 with that immediate.
#define TC_L(t)                                                                              \
    case 0x##t:                                                                              \
        asm("lop3.b32 %0, %1, %2, %3, 0x" #t ";" : "=r"(r) : "r"(x), "r"(y), "r"(z));        \
        break;
#define TC_L16(h)                                                                            \
    TC_L(h##0) TC_L(h##1) TC_L(h##2) TC_L(h##3) TC_L(h##4) TC_L(h##5) TC_L(h##6) TC_L(h##7)  \
    TC_L(h##8) TC_L(h##9) TC_L(h##a) TC_L(h##b) TC_L(h##c) TC_L(h##d) TC_L(h##e) TC_L(h##f)

__device__ __forceinline__ uint32_t lut3(uint32_t tt, uint32_t x, uint32_t y, uint32_t z)
{
    uint32_t r = 0;
    switch (tt) {
        TC_L16(0) TC_L16(1) TC_L16(2) TC_L16(3) TC_L16(4) TC_L16(5) TC_L16(6) TC_L16(7)
        TC_L16(8) TC_L16(9) TC_L16(a) TC_L16(b) TC_L16(c) TC_L16(d) TC_L16(e) TC_L16(f)
    }
    return r;
}

// One pass of a LUT job: every op reads three slots and writes one.
__device__ __forceinline__ void run_luts(char *Sb, const uint4 *ops, uint32_t n)
{
    uint4 next = n ? __ldg(ops) : make_uint4(0, 0, 0, 0);
    for (uint32_t i = 0; i < n; i++) {
        const uint4 op = next;
        if (i + 1 < n)
            next = __ldg(ops + i + 1);
        const uint32_t x = *(const uint32_t *)(Sb + op.x);
        const uint32_t y = *(const uint32_t *)(Sb + op.y);
        const uint32_t z = *(const uint32_t *)(Sb + op.z);
        *(uint32_t *)(Sb + (op.w & 0xffffffu)) = lut3(op.w >> 24, x, y, z);
    }
}

// 32 x 32 bit transpose: A[l] bit b -> A[b] bit l
__device__ __forceinline__ void transpose32(uint32_t *A)
{
#pragma unroll
    for (int j = 16, m0 = 0; j != 0; j >>= 1, m0++) {
        const uint32_t m = j == 16 ? 0x0000ffffu : j == 8 ? 0x00ff00ffu : j == 4 ? 0x0f0f0f0fu
                         : j == 2 ? 0x33333333u : 0x55555555u;
#pragma unroll
        for (int k = 0; k < 32; k = ((k | j) + 1) & ~j) {
            const uint32_t t = ((A[k] >> j) ^ A[k | j]) & m;
            A[k | j] ^= t;
            A[k] ^= t << j;
        }
    }
}

// The specification's right side for assignment x (src/spec.c:344-377).
__device__ uint64_t spec_value(const TcBatchJob &J, const TcBatchRpn *rpn, const uint8_t *vars,
                               uint64_t x, int width)
{
    uint64_t st[24];
    int sp = 0;
    for (uint32_t i = 0; i < J.nrpn; i++) {
        const uint32_t op = rpn[i].op;
        const uint64_t v = rpn[i].v;
        if (op == 0) {                    // TS_NUM
            st[sp++] = v;
        } else if (op == 1) {             // TS_VAR: bits of x
            const uint8_t *d = vars + 65 * v;
            uint64_t val = 0;
            for (int b = 0; b < d[0]; b++)
                val |= ((x >> d[1 + b]) & 1ull) << b;
            st[sp++] = val;
        } else if (op == 10) {            // TS_NOT
            st[sp - 1] = ~st[sp - 1];
        } else if (op == 11) {            // TS_NEG
            st[sp - 1] = 0ull - st[sp - 1];
        } else {
            const uint64_t b = st[--sp];
            uint64_t a = st[sp - 1];
            switch (op) {
            case 2: a += b; break;
            case 3: a -= b; break;
            case 4: a *= b; break;
            case 5: a &= b; break;
            case 6: a |= b; break;
            case 7: a ^= b; break;
            case 8: a = b < 64 ? a << b : 0; break;
            default: a = b < 64 ? a >> b : 0; break;
            }
            st[sp - 1] = a;
        }
    }
    return width == 64 ? st[0] : st[0] & ((1ull << width) - 1);
}

__global__ void __launch_bounds__(B) tc_batch_kernel(TcBatchDev d)
{
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t unit_s;
    __shared__ uint32_t masks[B];
    __shared__ unsigned long long block_hits;
    const uint32_t tid = threadIdx.x;
    uint32_t *S = smem + tid;
    for (;;) {
        if (tid == 0) {
            unit_s = d.unit_base + atomicAdd(d.next_unit, 1u);
            block_hits = 0;
        }
        __syncthreads();
        const uint32_t unit = unit_s;
        if (unit >= d.nunits)
            return;
        const TcBatchJob J = d.jobs[d.unit_job[unit]];
        const uint16_t *L = d.lists + J.lists;
        const uint64_t w0 = (uint64_t)(unit - J.first_unit) * J.unit_words;
        const uint64_t w1 = w0 + J.unit_words < J.words ? w0 + J.unit_words : J.words;
        uint32_t recorded = 0;  // meaningful in thread 0
        unsigned long long hits = 0;
        for (uint64_t base = w0; base < w1; base += B) {
            const uint64_t w = base + tid;
            const uint64_t x0 = w << 5;
            uint32_t valid = 0;
            if (w < w1)
                valid = J.space - x0 >= 32 ? 0xffffffffu : (1u << (uint32_t)(J.space - x0)) - 1u;
            const uint16_t *zero = L + 2 * J.n_in;
            if (J.lut) {
                S[0] = 0u;
                S[B] = 0xffffffffu;
                for (uint32_t k = 0; k < J.n_in; k++)
                    S[L[2 * k] * B] = lane_word(w, J.n_in - 1 - k);
                run_luts((char *)S, (const uint4 *)d.luts + J.code_a, J.nb_a);
            } else {
                // the power-on state: cleared cells, constants, inputs from the assignment number
                for (uint32_t z = 0; z < J.n_zero; z++)
                    S[zero[z] * B] = 0u;
                S[(J.one_a - 1u) * B] = 0u;  /* ZERO and ONE of each program */
                S[J.one_a * B] = 0xffffffffu;
                if (J.mode == EN_EQUIV) {
                    S[(J.one_b - 1u) * B] = 0u;
                    S[J.one_b * B] = 0xffffffffu;
                }
                for (uint32_t k = 0; k < J.n_in; k++) {
                    const uint32_t v = lane_word(w, J.n_in - 1 - k);
                    S[L[2 * k] * B] = v;
                    if (J.mode == EN_EQUIV)
                        S[L[2 * k + 1] * B] = v;
                }
                uint32_t r = 0;
                for (uint32_t t = 0; t < J.ticks; t++)
                    r = run_program(S, d.code + J.code_a, J.nb_a, r);
                if (J.mode == EN_EQUIV) {
                    uint32_t rb = 0;
                    for (uint32_t t = 0; t < J.ticks; t++)
                        rb = run_program(S, d.code + J.code_b, J.nb_b, rb);
                }
            }
            const uint16_t *cmp = zero + J.n_zero;
            uint32_t m = 0;
            if (J.mode == EN_EQUIV) {
                for (uint32_t o = 0; o < J.n_cmp; o++)
                    m |= S[cmp[2 * o] * B] ^ S[cmp[2 * o + 1] * B];
            } else if (J.mode == EN_SEARCH) {
                m = 0xffffffffu;
                for (uint32_t o = 0; o < J.n_cmp; o++) {
                    const uint32_t v = S[cmp[2 * o] * B];
                    m &= cmp[2 * o + 1] ? v : ~v;
                }
            } else {
                uint32_t lo[32], hi[32];
                for (int b = 0; b < 32; b++) {
                    lo[b] = b < (int)J.n_cmp ? S[cmp[b] * B] : 0u;
                    hi[b] = b + 32 < (int)J.n_cmp ? S[cmp[b + 32] * B] : 0u;
                }
                transpose32(lo);
                if (J.n_cmp > 32)
                    transpose32(hi);
                for (int l = 0; l < 32; l++) {
                    const uint64_t got = (uint64_t)lo[l] | ((uint64_t)hi[l] << 32);
                    const uint64_t want = spec_value(J, d.rpn + J.rpn, d.vars + J.vars, x0 + l,
                                                     (int)J.n_cmp);
                    m |= (uint32_t)(got != want) << l;
                }
            }
            m &= valid;
            hits += __popc(m);
            if (__syncthreads_or(m != 0u)) {
                masks[tid] = m;
                __syncthreads();
                if (tid == 0)
                    for (uint32_t t = 0; t < B && recorded < TC_BATCH_SHOW; t++)
                        for (uint32_t mm = masks[t]; mm && recorded < TC_BATCH_SHOW;
                             mm &= mm - 1u)
                            d.unit_hits[(size_t)unit * TC_BATCH_SHOW + recorded++] =
                                ((base + t) << 5) + (unsigned long long)(__ffs(mm) - 1);
                __syncthreads();
            }
        }
        for (int o = 16; o > 0; o >>= 1)
            hits += __shfl_xor_sync(0xffffffffu, hits, o);
        if ((tid & 31u) == 0 && hits)
            atomicAdd(&block_hits, hits);
        __syncthreads();
        if (tid == 0) {
            const uint32_t j = d.unit_job[unit];
            d.unit_count[unit] = recorded;
            if (block_hits)
                atomicAdd(d.hits + j, block_hits);
            // the last unit of a job publishes its result to the host: every unit's writes are
            // made visible system-wide before it counts itself finished
            __threadfence_system();
            if (atomicSub(d.remaining + j, 1u) == 1u) {
                __threadfence();
                d.hits_out[j] = atomicAdd(d.hits + j, 0ull);
                __threadfence_system();
                *(volatile uint32_t *)(d.done + j) = 1u;
            }
        }
        __syncthreads();
    }
}

extern "C" int tc_batch_launch(const TcBatchDev *d, int slots, cudaStream_t stream, double share,
                               int *grid_out, char *err, size_t errlen)
{
    const size_t smem = (size_t)slots * B * sizeof(uint32_t);
    if (!tc_cu_check(cudaFuncSetAttribute(tc_batch_kernel,
                                          cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                     "batch smem", err, errlen))
        return 0;
    int per_sm = 0;
    if (!tc_cu_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_batch_kernel, B,
                                                                   smem),
                     "batch occupancy", err, errlen))
        return 0;
    if (per_sm < 1)
        return tc_fail(err, errlen, "the batch needs %zu bytes of shared memory per block", smem);
    int grid = (int)(tc_engine.sms * per_sm * share);
    if ((uint32_t)grid > d->nunits - d->unit_base)
        grid = (int)(d->nunits - d->unit_base);
    if (grid < 1)
        grid = 1;
    *grid_out = grid;
    tc_batch_kernel<<<grid, B, smem, stream>>>(*d);
    return tc_cu_check(cudaGetLastError(), "batch launch", err, errlen);
}
