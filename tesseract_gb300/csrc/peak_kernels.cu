// The LOP3 issue-rate microbenchmark: the denominator of the engine's roofline.
//
// Every thread runs eight independent chains of 3-input LOP3 (explicit lop3.b32 in PTX, so the
// compiler can neither fold nor reorder them away); a full grid of them measures how many
// 32-bit logic operations per second the device's integer ALU pipes issue.  Each such operation
// is 32 one-bit lane operations.
#include <cuda_runtime.h>
#include <stdio.h>

#include "engine.h"

#define CHAINS 8
#define UNROLL 16

__global__ void __launch_bounds__(256) tc_lop3_peak_kernel(unsigned *sink, int iters)
{
    unsigned x[CHAINS];
    const unsigned y = threadIdx.x * 0x9E3779B9u, z = blockIdx.x * 0x85EBCA6Bu + 1u;
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        x[k] = threadIdx.x + 977u * (unsigned)k;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int u = 0; u < UNROLL; u++) {
#pragma unroll
            for (int k = 0; k < CHAINS; k++)
                asm volatile("lop3.b32 %0, %0, %1, %2, 0x96;" : "+r"(x[k]) : "r"(y), "r"(z));
        }
    }
    unsigned acc = 0;
#pragma unroll
    for (int k = 0; k < CHAINS; k++)
        acc ^= x[k];
    if (acc == 0x12345678u)  // practically never; keeps the chains live
        sink[blockIdx.x] = acc;
}

extern "C" int cuda_lop3_peak(double *ops_per_second, double *seconds, char *err, size_t errlen)
{
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tc_lop3_peak_kernel, 256, 0);
    if (per_sm < 1)
        per_sm = 1;
    unsigned blocks = (unsigned)(tc_engine.sms * per_sm);
    unsigned *sink = nullptr;
    if (!tc_cu_check(cudaMalloc(&sink, blocks * sizeof(unsigned)), "cudaMalloc", err, errlen))
        return 0;
    const int iters = 2048;
    cudaStream_t s = tc_engine.stream;
    tc_lop3_peak_kernel<<<blocks, 256, 0, s>>>(sink, 64);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; rep++) {
        cudaEventRecord(tc_engine.ev0, s);
        tc_lop3_peak_kernel<<<blocks, 256, 0, s>>>(sink, iters);
        cudaEventRecord(tc_engine.ev1, s);
        if (!tc_cu_check(cudaEventSynchronize(tc_engine.ev1), "tc_lop3_peak", err, errlen)) {
            cudaFree(sink);
            return 0;
        }
        float ms = 0;
        cudaEventElapsedTime(&ms, tc_engine.ev0, tc_engine.ev1);
        if (ms < best)
            best = ms;
    }
    cudaFree(sink);
    double ops = (double)blocks * 256.0 * iters * UNROLL * CHAINS;
    *seconds = best / 1e3;
    *ops_per_second = ops / *seconds;
    return 1;
}
