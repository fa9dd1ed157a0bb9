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
#define TC_PTX_BLOCK 128  /* threads per block of the kernels built from PTX written directly */
#define TC_MAX_KERNELS 8

typedef struct {
    void  *ptr;
    size_t bytes;
} TcBuf;

typedef struct {
    uint64_t hash;
    double   compile_seconds;  /* NVRTC and the module load */
    double   load_seconds;     /* the module load alone */
    size_t   cubin_bytes;
    int      regs, local_bytes, cached;
    /* generated enumeration kernels: the code generator's count of their work per word
       (TcGenWork); stretch_steps = 0 for other kernels */
    int      luts_per_step, luts_per_stretch, stretch_steps, compare_ops;
    int      block;  /* generated enumeration kernels: the threads per block they were made for */
    int      ptx;    /* built from PTX written directly (tc_module_build_ptx) */
    char     log[2048];
} TcModInfo;

typedef struct {
    cudaLibrary_t lib;
    cudaKernel_t  fn[TC_MAX_KERNELS];
    TcModInfo     info;
} TcModule;

/* A module compiled but not loaded (tc_module_build: NVRTC only, no CUDA call) */
typedef struct {
    char     *cubin;
    size_t    cubin_len;
    int       cached;  /* the module cache holds it already: nothing was compiled */
    TcModInfo info;
} TcBuilt;

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
/* tc_module in two steps: NVRTC (safe from any host thread, no CUDA call), then the load */
int    tc_module_build(const char *src, size_t len, const char *extra_opt, TcBuilt *b, char *err,
                       size_t errlen);
int    tc_module_load(const char *src, size_t len, TcBuilt *b, const char *const *kernels,
                      int nkernels, TcModule *out, char *err, size_t errlen);
/* tc_module_build for PTX text (ptxas through nvJitLink at -O0, or -O3 when opt is set); the
   module cache is keyed by the text as for CUDA C */
int    tc_module_build_ptx(const char *ptx, size_t len, int opt, TcBuilt *b, char *err,
                           size_t errlen);
/* Build modes of the generated enumeration kernels (engine.c says what each builds) */
enum { TC_BUILD_OPT, TC_BUILD_QUICK, TC_BUILD_QUICK_ONLY, TC_BUILD_SERVE };
/* 1 (default): quick-start builds of equivalence and search jobs write PTX directly (ptxgen.c)
   instead of CUDA C for NVRTC */
extern int tc_enum_ptx;
/* ptxas optimisation of a batch's PTX builds: 0 (default) or 3 */
extern int tc_enum_ptx_opt;
/* Is job e's quick-start build PTX written directly? */
int tc_enum_quick_ptx(const Enum *e);
/* cuda_enum_run's build mode (default TC_BUILD_OPT) */
extern int tc_enum_run_fast;
void   tc_built_free(TcBuilt *b);
int    tc_enum_prepare(const Enum *e, int *in_map, int *out_map, char *err, size_t errlen);
/* The loaded kernel of a job that an earlier enumeration compiled (the optimised build, or the
   quick one of build mode `fast`), else an error; allocates nothing (its maps are fixed buffers,
   so programs of more than TC_CACHED_MAX_OUTPUTS outputs are refused). */
#define TC_CACHED_MAX_OUTPUTS 4096
int    tc_enum_cached(const Enum *e, int fast, TcModule *m, char *err, size_t errlen);

/* One enumeration on the generated-kernel engine in steps, for callers that overlap many
   (serving): prepare (refusals, code generation, NVRTC and module load through the cache, the
   launch shape; no device work; safe from several host threads at once), launch on a stream into
   a caller's device workspace of tc_enum_job_ws_bytes (at most tc_enum_job_ws_max) with the
   workspace copied behind it into the caller's pinned host memory, and the result from that copy
   once the stream has passed it. */
typedef struct TcEnumPending TcEnumPending;
typedef struct {
    TcModule   m;
    uint64_t   words, space, per_warp, blocks, warps;
    uint32_t   parts, part, nsel;
    EnumResult base;     /* space, tried, ops */
    TcEnumPending *pending;  /* built by tc_enum_job_build, not yet loaded */
    int            pidx;     /* its kernel in the pending group */
} TcEnumJob;
/* fast: the build mode (TC_BUILD_*).  prepare = build (code generation and NVRTC or ptxas: no
   CUDA call) + load (the module load, which waits for the device's running work, and the launch
   shape); drop frees a build that will not be loaded. */
int    tc_enum_job_prepare(const Enum *e, TcEnumJob *j, int fast, char *err, size_t errlen);
int    tc_enum_job_build(const Enum *e, TcEnumJob *j, int fast, char *err, size_t errlen);
/* n (1..TC_MAX_KERNELS) jobs built together: their uncached kernels in one NVRTC program and,
   later, one module load */
int    tc_enum_jobs_build(const Enum *const *e, TcEnumJob *const *j, int n, int fast, char *err,
                          size_t errlen);
int    tc_enum_job_load(const Enum *e, TcEnumJob *j, char *err, size_t errlen);
void   tc_enum_job_drop(TcEnumJob *j);
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
