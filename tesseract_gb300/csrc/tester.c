/* Tester 1 on the GPU, the replacement of t1_run (src/tester.c:235-275): every random program
   (src/tester.c:57-81, seeded by t1_program_seed, src/tester.c:51-55) runs from 512 random
   states and the cycle length of every run goes into the size's histogram, as t1_work
   (src/tester.c:182-223) adds it up.  The programs of one size run as one launch of the
   tester kernel, one block each; sizes and chunks go in the reference's order (programs k = 0,
   1, ... of each size), so the histogram, the pass count and the longest cycle with its
   program are the reference's.  With a time limit (programs = 0) whole chunks run until the
   time is up: no program is cut off, so `unfinished` stays 0. */
#include <stdlib.h>
#include <string.h>

#include "engine.h"
#include "tester.h"

int tc_t1_launch(const TcT1Dev *d, uint32_t nprogs, uint32_t max_cells, cudaStream_t stream,
                 char *err, size_t errlen);

#define CHUNK 8192  /* programs per launch */

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

static int bucket(uint64_t lam)
{
    int b = 0;
    while (b < T1_BUCKETS - 2 && ((uint64_t)1 << b) < lam)
        b++;
    return b;
}

/* Programs k0 .. k0 + n - 1 of size cells: one launch; their results go into st. */
static int run_chunk(const T1Config *cfg, uint32_t cells, uint64_t k0, uint32_t n, T1Size *st,
                     char *err, size_t errlen)
{
    size_t len = program_len(cfg, cells);
    uint32_t ncells = cells + CELL_FIRST_FREE, writable = cells;
    uint32_t nsample = writable < 64 ? writable : 64;
    size_t code_n = (size_t)n * len, jobs_b = (size_t)n * sizeof(TcT1Job);
    size_t code_b = code_n * 4, sample_b = (size_t)nsample * 4;
    size_t lam_b = (size_t)n * 512 * 8, passes_b = (size_t)n * 8;
    TcT1Job *jobs = tc_xcalloc(n, sizeof *jobs);
    uint32_t *code = tc_xmalloc(code_b + 4), sample[64];
    for (uint32_t i = 0; i < nsample; i++)
        sample[i] = CELL_FIRST_FREE + (uint32_t)((uint64_t)i * writable / nsample);
    for (uint32_t i = 0; i < n; i++) {
        uint64_t ps = tc_t1_program_seed(cfg->seed, cells, k0 + i);
        Program p;
        tc_random_program(&p, cells, len, ps);
        for (size_t q = 0; q < len; q++)
            code[(size_t)i * len + q] = p.code[q].addr << 1 | p.code[q].op;
        tc_program_free(&p);
        jobs[i].seed = ps;
        jobs[i].ncells = ncells;
        jobs[i].len = (uint32_t)len;
        jobs[i].code = (uint32_t)((size_t)i * len);
        jobs[i].sample = 0;
        jobs[i].nsample = nsample;
    }
    size_t o_code = 0, o_jobs = (code_b + 255) & ~(size_t)255;
    size_t o_sample = o_jobs + ((jobs_b + 255) & ~(size_t)255);
    size_t o_lam = o_sample + 256, o_passes = o_lam + ((lam_b + 255) & ~(size_t)255);
    size_t total = o_passes + passes_b;
    char *dev = NULL;
    uint64_t *lam = tc_xmalloc(lam_b), *passes = tc_xmalloc(passes_b);
    cudaStream_t s = tc_engine.stream;
    TcT1Dev d;
    int ok = tc_cu_check(cudaMalloc((void **)&dev, total), "cudaMalloc", err, errlen);
    if (ok) {
        d.jobs = (const TcT1Job *)(dev + o_jobs);
        d.code = (const uint32_t *)(dev + o_code);
        d.sample = (const uint32_t *)(dev + o_sample);
        d.lam = (uint64_t *)(dev + o_lam);
        d.passes = (uint64_t *)(dev + o_passes);
        d.max_passes = cfg->max_passes;
        ok = tc_cu_check(cudaMemcpyAsync(dev + o_code, code, code_b, cudaMemcpyHostToDevice, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(dev + o_jobs, jobs, jobs_b, cudaMemcpyHostToDevice, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(dev + o_sample, sample, sample_b ? sample_b : 4,
                                         cudaMemcpyHostToDevice, s),
                         "copy", err, errlen) &&
             tc_t1_launch(&d, n, ncells, s, err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(lam, dev + o_lam, lam_b, cudaMemcpyDeviceToHost, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaMemcpyAsync(passes, dev + o_passes, passes_b,
                                         cudaMemcpyDeviceToHost, s),
                         "copy", err, errlen) &&
             tc_cu_check(cudaStreamSynchronize(s), "tester1", err, errlen);
    }
    if (dev)
        cudaFree(dev);
    for (uint32_t i = 0; ok && i < n; i++) {  /* as t1_work adds one program up */
        st->passes += passes[i];
        st->programs++;
        st->starts += 512;
        for (int l = 0; l < 512; l++) {
            uint64_t v = lam[(size_t)i * 512 + l];
            if (!v) {
                st->hist[T1_BUCKETS - 1]++;
                continue;
            }
            st->hist[bucket(v)]++;
            if (v > st->longest) {
                st->longest = v;
                st->longest_seed = jobs[i].seed;
            }
        }
    }
    free(lam);
    free(passes);
    free(jobs);
    free(code);
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
    double t0 = tc_now();
    uint64_t next[T1_SIZES] = {0};
    for (;;) {
        int any = 0;
        for (int si = 0; si < cfg->nsizes; si++) {
            uint64_t left = cfg->programs ? cfg->programs - next[si] : CHUNK;
            if (!left)
                continue;
            uint32_t n = left < CHUNK ? (uint32_t)left : CHUNK;
            if (!run_chunk(cfg, cfg->cells[si], next[si], n, &out[si], err, errlen))
                return -1;
            next[si] += n;
            any = 1;
        }
        if (!any || (!cfg->programs && tc_now() - t0 >= cfg->seconds))
            break;
    }
    return tc_now() - t0;
}
