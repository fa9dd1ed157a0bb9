/* The engine's runtime state and helpers shared by the host files (engine.c, cube.c, batch.c,
   serve.c, super.c). */
#ifndef TC_ENGINE_H
#define TC_ENGINE_H

#include <cuda_runtime_api.h>

#include "tc_host.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TC_ENUM_BLOCK 256
#define TC_MAX_KERNELS 8

typedef struct {
    void  *ptr;
    size_t bytes;
} TcBuf;

typedef struct {
    uint64_t hash;
    double   compile_seconds;
    size_t   cubin_bytes;
    int      regs, local_bytes, cached;
    /* generated enumeration kernels: the code generator's count of their work per word
       (TcGenWork); stretch_steps = 0 for other kernels */
    int      luts_per_step, luts_per_stretch, stretch_steps, compare_ops;
    int      block;  /* generated enumeration kernels: the threads per block they were made for */
    char     log[2048];
} TcModInfo;

typedef struct {
    cudaLibrary_t lib;
    cudaKernel_t  fn[TC_MAX_KERNELS];
    TcModInfo     info;
} TcModule;

typedef struct {
    int          ready;
    int          dev;
    cudaStream_t stream;
    cudaEvent_t  ev0, ev1;
    int       sms, cc_major, cc_minor, smem_optin;
    char      name[256];
    TcBuf     ws_hits, ws_list, ws_count;
    /* the last launch, for reports */
    TcModInfo last;
    float     last_kernel_ms;
    unsigned  last_grid, last_block;
} TcEngine;

extern TcEngine tc_engine;

static inline dim3 dim3u(unsigned x)
{
    dim3 d;
    d.x = x;
    d.y = 1;
    d.z = 1;
    return d;
}

double tc_now(void);
int    tc_fail(char *err, size_t errlen, const char *fmt, ...);
int    tc_cu_check(cudaError_t rc, const char *what, char *err, size_t errlen);
int    tc_scratch(TcBuf *b, size_t bytes, char *err, size_t errlen);
int    tc_module(const char *src, size_t len, const char *const *kernels, int nkernels,
                 const char *extra_opt, TcModule *out, char *err, size_t errlen);
int    tc_enum_prepare(const Enum *e, int *in_map, int *out_map, char *err, size_t errlen);
/* The loaded kernel of a job that an earlier enumeration compiled, else an error; allocates
   nothing (its maps are fixed buffers, so programs of more than TC_CACHED_MAX_OUTPUTS outputs
   are refused). */
#define TC_CACHED_MAX_OUTPUTS 4096
int    tc_enum_cached(const Enum *e, TcModule *m, char *err, size_t errlen);

/* One enumeration on the generated-kernel engine in steps, for callers that overlap many
   (serving): prepare (refusals, code generation, NVRTC and module load through the cache, the
   launch shape; no device work; safe from several host threads at once), launch on a stream into
   a caller's device workspace of tc_enum_job_ws_bytes (at most tc_enum_job_ws_max) with the
   workspace copied behind it into the caller's pinned host memory, and the result from that copy
   once the stream has passed it. */
typedef struct {
    TcModule   m;
    uint64_t   words, space, per_warp, blocks, warps;
    uint32_t   parts, part, nsel;
    EnumResult base;  /* space, tried, ops */
} TcEnumJob;
int    tc_enum_job_prepare(const Enum *e, TcEnumJob *j, char *err, size_t errlen);
size_t tc_enum_job_ws_bytes(const TcEnumJob *j);
size_t tc_enum_job_ws_max(void);
int    tc_enum_job_launch(const TcEnumJob *j, void *dev_ws, void *host_ws, cudaStream_t st,
                          char *err, size_t errlen);
void   tc_enum_job_result(const TcEnumJob *j, const void *host_ws, EnumResult *r);
void   tc_enum_shares(const Enum *e, uint64_t space, uint64_t *sel_chunks, uint64_t *tried,
                      uint64_t *passes_run);

#ifdef __cplusplus
}
#endif
#endif
