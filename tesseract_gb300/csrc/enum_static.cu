// cuda_enum_run_static: cuda_enum_run with its workspace in a fixed device array.
//
// cuda_enum_run keeps its workspace (the hit counter, each warp's first 16 hits and each warp's
// count of them) in device buffers that grow with cudaMalloc, after a cudaFree of the old ones,
// whenever a launch needs more warps than any before.  Two kinds of callers cannot allow that:
//   - a serving loop that has handed the device's memory out to admitted jobs by their
//     footprints: an allocation inside the call could fail, or take memory that admission
//     counted for a job already in flight;
//   - callers with kernels in flight on other streams: cudaFree waits for the whole device, so
//     growing the workspace would stall their work.
// This entry point calls no cudaMalloc, cudaFree or other allocating routine, on the device or
// on the host.  Its device workspace is tc_enum_scratch below, sized for TC_STATIC_WARPS warps;
// a launch that would need more warps is refused with an error.  The hit lists come back
// through a fixed buffer on the stack, TC_STATIC_RUN warps at a time, with stream-ordered copies
// on the engine's stream.  It compiles nothing either: the job's generated kernel must already
// be loaded by an earlier cuda_enum_run of the same job, else the call fails with an error.
//
// Set-up: the first call on a device, with that device current, takes the array's address with
// cudaGetSymbolAddress.  With CUDA's lazy module loading that first use loads this file's module
// (and so places the array), so make the first call before any stream capture.
//
// Every call shares the one array, which keeps the last call's contents.  Each call clears, on
// its stream, the hit counter and the per-warp counts it will use before its launch; the hit
// lists are read only up to those counts.  Calls that overlap on the GPU (two host threads
// calling at once) race on the array.
#include <cuda_runtime.h>
#include <stdlib.h>
#include <stdint.h>
#include <string.h>

#include "codegen.h"
#include "engine.h"

#define TC_STATIC_WARPS 16384u        // 16 hits of 8 bytes and one count per warp
#define TC_STATIC_LIST_OFF 256u
#define TC_STATIC_COUNT_OFF (TC_STATIC_LIST_OFF + TC_STATIC_WARPS * 16u * 8u)
#define TC_STATIC_BYTES (TC_STATIC_COUNT_OFF + TC_STATIC_WARPS * 4u)   // 2,162,944 bytes
#define TC_STATIC_DEVICES 64
#define TC_STATIC_RUN 128u            // warps whose hits come back per copy (16 KB on the stack)

// [0, 8): hit counter; [256, +2 MiB): hit lists; then the counts.
static __device__ __align__(256) unsigned char tc_enum_scratch[TC_STATIC_BYTES];

static void *scratch_at[TC_STATIC_DEVICES];

static int scratch_for_current_device(unsigned char **out, char *err, size_t errlen)
{
    int dev = -1;
    if (!tc_cu_check(cudaGetDevice(&dev), "cudaGetDevice", err, errlen))
        return 0;
    if (dev < 0 || dev >= TC_STATIC_DEVICES)
        return tc_fail(err, errlen, "cuda_enum_run_static: device %d is beyond the %d supported",
                       dev, TC_STATIC_DEVICES);
    if (!scratch_at[dev]) {
        void *p = NULL;
        if (!tc_cu_check(cudaGetSymbolAddress(&p, tc_enum_scratch), "cudaGetSymbolAddress", err,
                         errlen))
            return 0;
        scratch_at[dev] = p;
    }
    *out = (unsigned char *)scratch_at[dev];
    return 1;
}

extern "C" int cuda_enum_run_static(const Enum *e, EnumResult *r, char *err, size_t errlen)
{
    memset(r, 0, sizeof *r);
    if (!tc_engine.ready)
        return tc_fail(err, errlen, "cuda_enum_run_static: the engine is not started; run the "
                       "same job once through cuda_enum_run first");
    TcModule m;
    if (!tc_enum_cached(e, TC_BUILD_OPT, &m, err, errlen))
        return 0;
    if (!cuda_engine_init(0, err, errlen))  // started already: makes its device current
        return 0;
    unsigned char *ws;
    if (!scratch_for_current_device(&ws, err, errlen))
        return 0;

    uint64_t space = 1ull << e->a->ninputs, sel, tried, pruns;
    tc_enum_shares(e, space, &sel, &tried, &pruns);
    r->space = space;
    r->tried = tried;
    r->ops = pruns * 512 * e->ticks * (e->a->len + (e->mode == EN_EQUIV ? e->b->len : 0));

    int per_sm = 0;
    const int block = m.info.block;  // the kernel's own block size (the autotuner may change it)
    if (!tc_cu_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, (const void *)m.fn[0],
                                                                     block, 0),
                     "occupancy", err, errlen))
        return 0;
    if (per_sm < 1)
        per_sm = 1;
    uint64_t words = sel * 1024;
    uint64_t blocks = (uint64_t)tc_engine.sms * (uint64_t)per_sm;
    uint64_t warps_needed = (words + 31) / 32;
    uint64_t max_blocks = (warps_needed + block / 32 - 1) / (block / 32);
    if (blocks > max_blocks)
        blocks = max_blocks ? max_blocks : 1;
    uint64_t warps = blocks * (uint64_t)(block / 32);
    if (warps > TC_STATIC_WARPS)
        return tc_fail(err, errlen, "cuda_enum_run_static: the launch needs %llu warps of hit "
                       "lists; the static workspace holds %u", (unsigned long long)warps,
                       TC_STATIC_WARPS);
    uint64_t per_warp = (words + warps - 1) / warps;
    per_warp = (per_warp + 31) / 32 * 32;
    if (!per_warp)
        per_warp = 32;

    cudaStream_t st = tc_engine.stream;
    TcEnumArgs args;  // the generated kernel's own argument block (codegen.h)
    memset(&args, 0, sizeof args);
    args.words = words;
    args.space = space;
    args.per_warp = per_warp;
    args.parts = (uint32_t)e->parts;
    args.part = (uint32_t)e->part;
    args.nsel = (uint32_t)(e->part_end - e->part + 1);
    args.hits = (uint64_t *)ws;
    args.list = (uint64_t *)(ws + TC_STATIC_LIST_OFF);
    args.count = (uint32_t *)(ws + TC_STATIC_COUNT_OFF);
    void *params[] = {&args};
    if (!tc_cu_check(cudaMemsetAsync(args.hits, 0, 8, st), "memset", err, errlen) ||
        !tc_cu_check(cudaMemsetAsync(args.count, 0, warps * 4, st), "memset", err, errlen) ||
        !tc_cu_check(cudaEventRecord(tc_engine.ev0, st), "event", err, errlen) ||
        !tc_cu_check(cudaLaunchKernel((const void *)m.fn[0], dim3u((unsigned)blocks),
                                      dim3u((unsigned)block), params, 0, st),
                     "launch tc_enum", err, errlen) ||
        !tc_cu_check(cudaEventRecord(tc_engine.ev1, st), "event", err, errlen))
        return 0;
    uint64_t hits = 0;
    if (!tc_cu_check(cudaMemcpyAsync(&hits, args.hits, 8, cudaMemcpyDeviceToHost, st), "hits",
                     err, errlen) ||
        !tc_cu_check(cudaStreamSynchronize(st), "tc_enum", err, errlen))
        return 0;
    // Every warp's hits (a kernel whose enumeration order is permuted does not find the
    // smallest in the first warps).  Counts and lists come over in runs of TC_STATIC_RUN warps,
    // on the engine's stream; only the counts this call cleared and its kernel wrote are read.
    uint32_t count[TC_STATIC_RUN];
    uint64_t got[TC_STATIC_RUN * 16];
    for (uint64_t w0 = 0; hits && w0 < warps; w0 += TC_STATIC_RUN) {
        uint64_t n = warps - w0 < TC_STATIC_RUN ? warps - w0 : TC_STATIC_RUN;
        if (!tc_cu_check(cudaMemcpyAsync(count, args.count + w0, n * 4, cudaMemcpyDeviceToHost,
                                         st),
                         "hit counts", err, errlen) ||
            !tc_cu_check(cudaMemcpyAsync(got, args.list + w0 * 16, n * 16 * 8,
                                         cudaMemcpyDeviceToHost, st),
                         "hits", err, errlen) ||
            !tc_cu_check(cudaStreamSynchronize(st), "hit copy", err, errlen))
            return 0;
        for (uint64_t i = 0; i < n; i++)
            for (uint32_t k = 0; k < count[i] && k < 16; k++)
                cuda_enum_add_hit(r, got[i * 16 + k]);
    }
    float ms = 0;
    cudaEventElapsedTime(&ms, tc_engine.ev0, tc_engine.ev1);
    r->seconds = ms / 1e3;
    r->hits = hits;
    r->threads = (int)(blocks * (uint64_t)block);
    tc_engine.last = m.info;
    tc_engine.last_kernel_ms = ms;
    tc_engine.last_grid = (unsigned)blocks;
    tc_engine.last_block = (unsigned)block;
    return 1;
}
