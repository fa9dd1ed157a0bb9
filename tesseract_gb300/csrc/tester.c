/* Tester 1 on the GPU, the replacement of t1_run (src/tester.c:235-275): every random program
   (src/tester.c:57-81, seeded by t1_program_seed, src/tester.c:51-55) runs from 512 random
   states and the cycle length of every run goes into the size's histogram, as t1_work
   (src/tester.c:182-223) adds it up.  The programs of one size run as one launch of the
   tester kernel, one block each, which makes its program and its starting states itself and adds
   its runs to the size's histogram on the device; the host only adds up the passes and finds
   the first program with the longest cycle, in the reference's order (programs k = 0, 1, ... of
   each size), so the histogram, the pass count and the longest cycle with its program are the
   reference's.  With a time limit (programs = 0) whole chunks run until the
   time is up: no program is cut off, so `unfinished` stays 0. */
#include <stdlib.h>
#include <string.h>

#include "engine.h"
#include "tester.h"

int tc_t1_launch(const TcT1Dev *d, uint32_t nprogs, cudaStream_t stream, char *err,
                 size_t errlen);

#define CHUNK 65536  /* programs per launch */

uint64_t tc_t1_program_seed(uint64_t seed, uint32_t cells, uint64_t k)
{
    uint64_t s = seed ^ ((uint64_t)cells << 40) ^ (k * 0xD1B54A32D192ED03ull);
    return tc_splitmix64(&s);
}

static size_t program_len(const T1Config *cfg, uint32_t cells)
{
    size_t len = (size_t)(cells * cfg->ratio + 0.5);
    return len ? len : 1;
}

/* Device buffers of one run: the histogram, then passes and longest cycle per program. */
typedef struct {
    uint64_t *dev, *hist, *passes, *longest;
} Bufs;

/* Programs k0 .. k0 + n - 1 of size cells: one launch; their results go into st. */
static int run_chunk(const T1Config *cfg, const Bufs *b, uint32_t cells, uint64_t k0, uint32_t n,
                     T1Size *st, char *err, size_t errlen)
{
    size_t len = program_len(cfg, cells);
    if (len > 0xffffffffu)
        return tc_fail(err, errlen, "%zu instructions per program: too many", len);
    TcT1Dev d;
    memset(&d, 0, sizeof d);
    d.seed = cfg->seed;
    d.k0 = k0;
    d.max_passes = cfg->max_passes;
    d.cells = cells;
    d.len = (uint32_t)len;
    d.nsample = cells < 64 ? cells : 64;
    d.hist = b->hist;
    d.passes = b->passes;
    d.longest = b->longest;
    uint64_t hist[T1_BUCKETS];
    uint64_t *passes = tc_xmalloc((size_t)n * 8), *longest = tc_xmalloc((size_t)n * 8);
    cudaStream_t s = tc_engine.stream;
    int ok = tc_cu_check(cudaMemsetAsync(b->hist, 0, sizeof hist, s), "memset", err, errlen) &&
             tc_t1_launch(&d, n, s, err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(hist, b->hist, sizeof hist, cudaMemcpyDeviceToHost, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(passes, b->passes, (size_t)n * 8,
                                         cudaMemcpyDeviceToHost, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(longest, b->longest, (size_t)n * 8,
                                         cudaMemcpyDeviceToHost, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaStreamSynchronize(s), "tester1", err, errlen);
    if (ok) {
        /* as t1_work adds each program up, in program order: the first longest cycle wins */
        for (int i = 0; i < T1_BUCKETS; i++)
            st->hist[i] += hist[i];
        for (uint32_t i = 0; i < n; i++) {
            st->passes += passes[i];
            st->programs++;
            st->starts += 512;
            if (longest[i] > st->longest) {
                st->longest = longest[i];
                st->longest_seed = tc_t1_program_seed(cfg->seed, cells, k0 + i);
            }
        }
    }
    free(passes);
    free(longest);
    return ok;
}

double cuda_t1_run(const T1Config *cfg, T1Size *out, int *threads, char *err, size_t errlen)
{
    *threads = 1;
    if (cfg->nsizes < 1 || cfg->nsizes > T1_SIZES || cfg->ratio <= 0 || cfg->max_passes == 0 ||
        (cfg->programs == 0 && cfg->seconds <= 0)) {
        tc_fail(err, errlen, "--ratio, --max-passes and --programs or --seconds must be positive");
        return -1;
    }
    if (!cuda_engine_init(0, err, errlen))
        return -1;
    memset(out, 0, (size_t)cfg->nsizes * sizeof *out);
    for (int si = 0; si < cfg->nsizes; si++) {
        out[si].cells = cfg->cells[si];
        out[si].len = program_len(cfg, cfg->cells[si]);
    }
    Bufs b;
    memset(&b, 0, sizeof b);
    if (!tc_cu_check(cudaMalloc((void **)&b.dev, (T1_BUCKETS + 2 * (size_t)CHUNK) * 8),
                     "cudaMalloc", err, errlen))
        return -1;
    b.hist = b.dev;
    b.passes = b.dev + T1_BUCKETS;
    b.longest = b.passes + CHUNK;
    double t0 = tc_now();
    uint64_t next[T1_SIZES] = {0};
    uint32_t chunk = cfg->programs ? CHUNK : 16384;  /* timed runs check the clock more often */
    int ok = 1;
    for (;;) {
        int any = 0;
        for (int si = 0; si < cfg->nsizes && ok; si++) {
            uint64_t left = cfg->programs ? cfg->programs - next[si] : chunk;
            if (!left)
                continue;
            uint32_t n = left < chunk ? (uint32_t)left : chunk;
            ok = run_chunk(cfg, &b, cfg->cells[si], next[si], n, &out[si], err, errlen);
            next[si] += n;
            any = 1;
        }
        if (!ok || !any || (!cfg->programs && tc_now() - t0 >= cfg->seconds))
            break;
    }
    cudaFree(b.dev);
    return ok ? tc_now() - t0 : -1;
}
