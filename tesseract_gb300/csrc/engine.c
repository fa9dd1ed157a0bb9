/* The engine's runtime: device set-up, NVRTC compilation with a content-addressed module cache,
   and cuda_enum_run (verify / equiv / search over every assignment).

   One process, one GPU, the primary context; all work goes to one engine stream.  Generated
   modules are compiled for the device's own architecture (sm_103a on GB300) and kept for the
   life of the process, keyed by the full text of the generated source. */
#include <cuda_runtime_api.h>
#include <nvJitLink.h>
#include <nvrtc.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "codegen.h"
#include "engine.h"

TcEngine tc_engine;
static pthread_mutex_t engine_lock = PTHREAD_MUTEX_INITIALIZER;

double tc_now(void)
{
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

int tc_fail(char *err, size_t errlen, const char *fmt, ...)
{
    if (err && errlen) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(err, errlen, fmt, ap);
        va_end(ap);
    }
    return 0;
}

int tc_cu_check(cudaError_t rc, const char *what, char *err, size_t errlen)
{
    if (rc == cudaSuccess)
        return 1;
    return tc_fail(err, errlen, "CUDA error in %s: %s (%s)", what, cudaGetErrorName(rc),
                   cudaGetErrorString(rc));
}

#define CU(call, what)                                               \
    do {                                                             \
        if (!tc_cu_check((call), (what), err, errlen))               \
            goto fail;                                               \
    } while (0)

int cuda_engine_init(int device, char *err, size_t errlen)
{
    pthread_mutex_lock(&engine_lock);
    if (tc_engine.ready) {
        int ok = cudaSetDevice(tc_engine.dev) == cudaSuccess;
        pthread_mutex_unlock(&engine_lock);
        return ok ? 1 : tc_fail(err, errlen, "cannot make the engine's device current");
    }
    struct cudaDeviceProp prop;
    int count = 0;
    CU(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (device < 0 || device >= count) {
        tc_fail(err, errlen, "no CUDA device %d (%d present)", device, count);
        goto fail;
    }
    CU(cudaSetDevice(device), "cudaSetDevice");
    CU(cudaGetDeviceProperties(&prop, device), "cudaGetDeviceProperties");
    tc_engine.dev = device;
    tc_engine.sms = prop.multiProcessorCount;
    tc_engine.cc_major = prop.major;
    tc_engine.cc_minor = prop.minor;
    tc_engine.smem_optin = (int)prop.sharedMemPerBlockOptin;
    snprintf(tc_engine.name, sizeof tc_engine.name, "%s", prop.name);
    CU(cudaStreamCreateWithFlags(&tc_engine.stream, cudaStreamNonBlocking), "cudaStreamCreate");
    CU(cudaEventCreate(&tc_engine.ev0), "cudaEventCreate");
    CU(cudaEventCreate(&tc_engine.ev1), "cudaEventCreate");
    tc_engine.ready = 1;
    pthread_mutex_unlock(&engine_lock);
    return 1;
fail:
    pthread_mutex_unlock(&engine_lock);
    return 0;
}

int cuda_device_info(char *buf, size_t len)
{
    char err[256];
    if (!cuda_engine_init(0, err, sizeof err)) {
        snprintf(buf, len, "%s", err);
        return 0;
    }
    snprintf(buf, len, "%s, %d SMs, sm_%d%d", tc_engine.name, tc_engine.sms, tc_engine.cc_major,
             tc_engine.cc_minor);
    return 1;
}

int cuda_last_launch(CudaLaunchStats *s)
{
    memset(s, 0, sizeof *s);
    s->kernel_ms = tc_engine.last_kernel_ms;
    s->regs = tc_engine.last.regs;
    s->local_bytes = tc_engine.last.local_bytes;
    s->grid = tc_engine.last_grid;
    s->block = tc_engine.last_block;
    s->compile_seconds = tc_engine.last.cached ? 0 : tc_engine.last.compile_seconds;
    s->cached = tc_engine.last.cached;
    const TcModInfo *m = &tc_engine.last;
    s->luts_per_step = m->luts_per_step;
    s->luts_per_stretch = m->luts_per_stretch;
    s->stretch_steps = m->stretch_steps;
    s->compare_ops = m->compare_ops;
    s->logic_ops_per_word = m->stretch_steps && m->compare_ops >= 0
                                ? m->luts_per_step + (double)m->luts_per_stretch /
                                  m->stretch_steps + m->compare_ops
                                : 0;
    s->ptx = m->ptx;
    return tc_engine.ready;
}

/* ---- workspace ------------------------------------------------------------------------------- */

int tc_scratch(TcBuf *b, size_t bytes, char *err, size_t errlen)
{
    if (b->bytes >= bytes)
        return 1;
    if (b->ptr)
        cudaFree(b->ptr);
    b->ptr = NULL;
    b->bytes = 0;
    if (!tc_cu_check(cudaMalloc(&b->ptr, bytes ? bytes : 16), "cudaMalloc", err, errlen))
        return 0;
    b->bytes = bytes;
    return 1;
}

/* ---- NVRTC and the module cache -------------------------------------------------------------- */

typedef struct {
    char     *src;
    size_t    len;
    cudaLibrary_t lib;
    TcModInfo     info;
} CacheEntry;

static CacheEntry *cache;
static size_t ncache, capcache;

static uint64_t text_hash(const char *s, size_t n)
{
    uint64_t h = 0xcbf29ce484222325ull;
    for (size_t i = 0; i < n; i++)
        h = (h ^ (unsigned char)s[i]) * 0x100000001b3ull;
    return h;
}

/* Finds src in the module cache (1: *out filled). */
static int cache_find(const char *src, size_t len, uint64_t h, TcModule *out)
{
    int found = 0;
    pthread_mutex_lock(&engine_lock);
    for (size_t i = 0; i < ncache && !found; i++)
        if (cache[i].info.hash == h && cache[i].len == len && !memcmp(cache[i].src, src, len)) {
            out->lib = cache[i].lib;
            out->info = cache[i].info;
            out->info.cached = 1;
            found = 1;
        }
    pthread_mutex_unlock(&engine_lock);
    return found;
}

void tc_built_free(TcBuilt *b)
{
    free(b->cubin);
    memset(b, 0, sizeof *b);
}

/* NVRTC on src, with no CUDA call: b gets the cubin (or cached = 1 when the module cache holds
   this source already). */
int tc_module_build(const char *src, size_t len, const char *extra_opt, TcBuilt *b, char *err,
                    size_t errlen)
{
    memset(b, 0, sizeof *b);
    b->info.hash = text_hash(src, len);
    TcModule m;
    if (cache_find(src, len, b->info.hash, &m)) {
        b->cached = 1;
        return 1;
    }
    double t0 = tc_now();
    nvrtcProgram prog;
    nvrtcResult nr = nvrtcCreateProgram(&prog, src, "tesseract_gen.cu", 0, NULL, NULL);
    if (nr != NVRTC_SUCCESS)
        return tc_fail(err, errlen, "NVRTC: %s", nvrtcGetErrorString(nr));
    char arch[64];
    snprintf(arch, sizeof arch, "--gpu-architecture=sm_%d%da", tc_engine.cc_major,
             tc_engine.cc_minor);
    const char *opts[8];
    int nopt = 0;
    opts[nopt++] = arch;
    opts[nopt++] = "--std=c++17";
    opts[nopt++] = "-lineinfo";
    opts[nopt++] = "--ptxas-options=-v";
    /* ptxas -O2 rather than its default -O3: measured on the GB300, the kernels run the
       same (mul16's verify 7.89 ms either way in alternating runs, cube Life 71,900 gen/s
       either way) and compiling takes ~35 % less (0.77 against 1.18 s for a
       20,000-instruction program); -O1 compiles faster still but runs Life 11 % slower */
    if (!(extra_opt && strstr(extra_opt, "--ptxas-options=-O")))
        opts[nopt++] = "--ptxas-options=-O2";
    if (extra_opt && *extra_opt)
        opts[nopt++] = extra_opt;
    nr = nvrtcCompileProgram(prog, nopt, opts);
    size_t loglen = 0;
    nvrtcGetProgramLogSize(prog, &loglen);
    char *log = tc_xmalloc(loglen + 1);
    log[0] = '\0';
    if (loglen)
        nvrtcGetProgramLog(prog, log);
    if (nr != NVRTC_SUCCESS) {
        tc_fail(err, errlen, "NVRTC compile failed: %s: %.400s", nvrtcGetErrorString(nr), log);
        free(log);
        nvrtcDestroyProgram(&prog);
        return 0;
    }
    nvrtcGetCUBINSize(prog, &b->cubin_len);
    b->cubin = tc_xmalloc(b->cubin_len + 1);
    nvrtcGetCUBIN(prog, b->cubin);
    nvrtcDestroyProgram(&prog);
    b->info.compile_seconds = tc_now() - t0;
    b->info.cubin_bytes = b->cubin_len;
    snprintf(b->info.log, sizeof b->info.log, "%s", log);
    free(log);
    return 1;
}

int tc_module_build_ptx(const char *ptx, size_t len, int opt, TcBuilt *b, char *err,
                        size_t errlen)
{
    memset(b, 0, sizeof *b);
    b->info.hash = text_hash(ptx, len);
    TcModule m;
    if (cache_find(ptx, len, b->info.hash, &m)) {
        b->cached = 1;
        return 1;
    }
    double t0 = tc_now();
    char arch[32];
    snprintf(arch, sizeof arch, "-arch=sm_%d%da", tc_engine.cc_major, tc_engine.cc_minor);
    const char *opts[] = {arch, opt ? "-O3" : "-O0"};
    nvJitLinkHandle h;
    nvJitLinkResult r = nvJitLinkCreate(&h, 2, opts);
    if (r != NVJITLINK_SUCCESS)
        return tc_fail(err, errlen, "nvJitLinkCreate: error %d", (int)r);
    r = nvJitLinkAddData(h, NVJITLINK_INPUT_PTX, ptx, len, "tesseract_gen.ptx");
    if (r == NVJITLINK_SUCCESS)
        r = nvJitLinkComplete(h);
    if (r == NVJITLINK_SUCCESS)
        r = nvJitLinkGetLinkedCubinSize(h, &b->cubin_len);
    if (r == NVJITLINK_SUCCESS) {
        b->cubin = tc_xmalloc(b->cubin_len + 1);
        r = nvJitLinkGetLinkedCubin(h, b->cubin);
    }
    if (r != NVJITLINK_SUCCESS) {
        size_t n = 0;
        char log[512] = "";
        if (nvJitLinkGetErrorLogSize(h, &n) == NVJITLINK_SUCCESS && n > 0) {
            char *full = tc_xmalloc(n + 1);
            if (nvJitLinkGetErrorLog(h, full) == NVJITLINK_SUCCESS)
                snprintf(log, sizeof log, "%s", full);
            free(full);
        }
        nvJitLinkDestroy(&h);
        tc_built_free(b);
        return tc_fail(err, errlen, "nvJitLink on generated PTX: error %d: %s", (int)r, log);
    }
    nvJitLinkDestroy(&h);
    b->info.ptx = 1;
    b->info.compile_seconds = tc_now() - t0;
    b->info.cubin_bytes = b->cubin_len;
    return 1;
}

/* Loads a built module (into the module cache) and finds its kernels; frees b's cubin.  With lazy
   loading the module reaches the device at the first query of a kernel, here.  Loading waits for
   the device's running work (it synchronises the context). */
int tc_module_load(const char *src, size_t len, TcBuilt *b, const char *const *kernels,
                   int nkernels, TcModule *out, char *err, size_t errlen)
{
    double tf = tc_now();
    if (!cache_find(src, len, b->info.hash, out)) {
        if (b->cached)
            return tc_fail(err, errlen, "module cache: a built module went missing");
        cudaLibrary_t lib;
        cudaError_t rc = cudaLibraryLoadData(&lib, b->cubin, NULL, NULL, 0, NULL, NULL, 0);
        if (!tc_cu_check(rc, "cudaLibraryLoadData", err, errlen)) {
            tc_built_free(b);
            return 0;
        }
        TcModInfo info = b->info;
        pthread_mutex_lock(&engine_lock);
        if (ncache == capcache) {
            capcache = capcache ? 2 * capcache : 16;
            cache = tc_xrealloc(cache, capcache * sizeof *cache);
        }
        cache[ncache].src = tc_xmalloc(len + 1);
        memcpy(cache[ncache].src, src, len);
        cache[ncache].src[len] = '\0';
        cache[ncache].len = len;
        cache[ncache].lib = lib;
        cache[ncache].info = info;
        ncache++;
        pthread_mutex_unlock(&engine_lock);
        out->lib = lib;
        out->info = info;
    }
    tc_built_free(b);
    for (int k = 0; k < nkernels && k < TC_MAX_KERNELS; k++) {
        if (!tc_cu_check(cudaLibraryGetKernel(&out->fn[k], out->lib, kernels[k]),
                         "cudaLibraryGetKernel", err, errlen))
            return 0;
        struct cudaFuncAttributes fa;
        if (k == 0 && cudaFuncGetAttributes(&fa, (const void *)out->fn[k]) == cudaSuccess) {
            out->info.regs = fa.numRegs;
            out->info.local_bytes = (int)fa.localSizeBytes;
        }
    }
    out->info.load_seconds = tc_now() - tf;
    if (!out->info.cached)
        out->info.compile_seconds += out->info.load_seconds;
    return 1;
}

int tc_module(const char *src, size_t len, const char *const *kernels, int nkernels,
              const char *extra_opt, TcModule *out, char *err, size_t errlen)
{
    TcBuilt b;
    return tc_module_build(src, len, extra_opt, &b, err, errlen) &&
           tc_module_load(src, len, &b, kernels, nkernels, out, err, errlen);
}

/* ---- verify / equiv / search ---------------------------------------------------------------- */

/* Keeps hit[0..nhit) the EN_SHOW smallest hits seen, ascending (the contract of enum_add_hit,
   src/enum.c:31-46): x goes after the hits not above it, and the largest falls off a full list. */
void cuda_enum_add_hit(EnumResult *r, uint64_t x)
{
    int n = r->nhit;
    if (n == EN_SHOW && x >= r->hit[EN_SHOW - 1])
        return;
    int lo = 0, hi = n;  /* the first hit above x */
    while (lo < hi) {
        int mid = (lo + hi) / 2;
        if (r->hit[mid] > x)
            hi = mid;
        else
            lo = mid + 1;
    }
    int kept = n < EN_SHOW ? n : EN_SHOW - 1;
    memmove(&r->hit[lo + 1], &r->hit[lo], (size_t)(kept - lo) * sizeof r->hit[0]);
    r->hit[lo] = x;
    r->nhit = kept + 1;
}

/* Adds one share's result into a total, as merge_raw does with --raw lines
   (src/work.c:341-371): counts add up, the slowest share's seconds, the 16 smallest hits. */
void cuda_enum_merge(EnumResult *into, const EnumResult *part)
{
    into->space = part->space;
    into->tried += part->tried;
    into->hits += part->hits;
    into->ops += part->ops;
    into->threads += part->threads;
    if (part->seconds > into->seconds)
        into->seconds = part->seconds;
    for (int i = 0; i < part->nhit; i++)
        cuda_enum_add_hit(into, part->hit[i]);
}

/* map[i] = the position in lb of the cell named like la[i] (names compare without case; the
   last of equal names wins), for lists of equal length (enum_match, src/enum.c:48-78). */
static int match_names(const Program *a, const uint32_t *la, size_t na, const Program *b,
                       const uint32_t *lb, size_t nb, int *map, const char *what, char *err,
                       size_t errlen)
{
    if (na != nb)
        return tc_fail(err, errlen, "the programs have %zu and %zu %s", na, nb, what);
    for (size_t i = 0; i < na; i++) {
        const char *name = a->cell_names[la[i]];
        size_t j = nb;
        while (j > 0 && !tc_same_name(b->cell_names[lb[j - 1]], name))
            j--;
        if (!j)
            return tc_fail(err, errlen, "the second program has no %s called %s",
                           what[0] == 'i' ? "input" : "output", name);
        map[i] = (int)(j - 1);
    }
    return 1;
}

/* The refusals of enum_run (src/enum.c:247-260) and the name matching of enum_match
   (src/enum.c:48-78).  in_map/out_map get n and noutputs entries. */
int tc_enum_prepare(const Enum *e, int *in_map, int *out_map, char *err, size_t errlen)
{
    if (e->a->special || (e->mode == EN_EQUIV && e->b->special))
        return tc_fail(err, errlen, "id and link cells connect the lanes, but every input needs "
                                    "a lane of its own here");
    if (e->a->ninputs > EN_MAX_IN)
        return tc_fail(err, errlen, "%zu inputs is too many to try them all (at most %d)",
                       e->a->ninputs, EN_MAX_IN);
    if (e->parts < 1 || e->part < 0 || e->part > e->part_end || e->part_end >= e->parts ||
        e->ticks < 1)
        return tc_fail(err, errlen, "bad --part or --ticks");
    if (e->mode != EN_EQUIV && !e->spec)
        return tc_fail(err, errlen, "%s needs a specification",
                       e->mode == EN_VERIFY ? "verify" : "search");
    if (e->mode == EN_EQUIV)
        return match_names(e->a, e->a->inputs, e->a->ninputs, e->b, e->b->inputs, e->b->ninputs,
                           in_map, "inputs", err, errlen) &&
               match_names(e->a, e->a->outputs, e->a->noutputs, e->b, e->b->outputs,
                           e->b->noutputs, out_map, "outputs", err, errlen);
    return 1;
}

/* What a share selection covers: chunks of 64 passes of 512 assignments (src/enum.c:11,
   215-242).  Fills selected chunks, assignments tried and passes run. */
void tc_enum_shares(const Enum *e, uint64_t space, uint64_t *sel_chunks, uint64_t *tried,
                    uint64_t *passes_run)
{
    uint64_t passes = (space + 511) / 512, nchunks = (passes + 63) / 64;
    uint64_t parts = (uint64_t)e->parts, sel = 0, lanes = 0, pruns = 0;
    uint64_t last = nchunks - 1;
    uint64_t last_lanes = space - last * 32768, last_passes = passes - last * 64;
    for (uint64_t r = (uint64_t)e->part; r <= (uint64_t)e->part_end; r++) {
        if (r >= nchunks)
            continue;
        uint64_t count = (nchunks - r + parts - 1) / parts;  /* c = r, r + parts, ... < nchunks */
        sel += count;
        int has_last = (last % parts) == r;
        lanes += (count - (uint64_t)has_last) * 32768 + (has_last ? last_lanes : 0);
        pruns += (count - (uint64_t)has_last) * 64 + (has_last ? last_passes : 0);
    }
    *sel_chunks = sel;
    *tried = lanes;
    *passes_run = pruns;
}

typedef struct {
    int       *in_map, *out_map;
    uint32_t  *b_in;
    TcGenEnum  g;
} EnumPlan;

static void plan_free(EnumPlan *pl)
{
    free(pl->in_map);
    free(pl->out_map);
    free(pl->b_in);
    memset(pl, 0, sizeof *pl);
}

/* The code generator's input for one enumeration, into maps the caller gave pl (in_map and b_in
   of ninputs + 1 entries, out_map of noutputs + 1), after the refusals and the name matching. */
static int plan_fill(const Enum *e, EnumPlan *pl, char *err, size_t errlen)
{
    size_t n = e->a->ninputs;
    if (!tc_enum_prepare(e, pl->in_map, pl->out_map, err, errlen))
        return 0;
    TcGenEnum *g = &pl->g;
    g->mode = e->mode;
    g->a = e->a;
    g->spec = (const TcSpec *)e->spec;
    g->ticks = e->ticks;
    g->block = TC_ENUM_BLOCK;
    if (e->mode == EN_EQUIV) {
        for (size_t k = 0; k < n; k++)
            pl->b_in[k] = e->b->inputs[pl->in_map[k]];
        g->b = e->b;
        g->b_inputs = pl->b_in;
        g->out_map = pl->out_map;
    }
    if (e->mode == EN_SEARCH)
        g->target = cuda_spec_value(e->spec, 0);
    return 1;
}

/* Refusals, name matching and the code generator's input for one enumeration (maps on the
   heap; plan_free releases them). */
static int plan_enum(const Enum *e, EnumPlan *pl, char *err, size_t errlen)
{
    memset(pl, 0, sizeof *pl);
    if (!e || !e->a)
        return tc_fail(err, errlen, "no program");
    size_t n = e->a->ninputs;
    pl->in_map = tc_xcalloc(n + 1, sizeof *pl->in_map);
    pl->out_map = tc_xcalloc(e->a->noutputs + 1, sizeof *pl->out_map);
    pl->b_in = tc_xcalloc(n + 1, sizeof *pl->b_in);
    if (!plan_fill(e, pl, err, errlen)) {
        plan_free(pl);
        return 0;
    }
    return 1;
}

/* ---- the generated-kernel cache, keyed by what the code generator reads ---------------------- */

typedef struct {
    uint64_t h1, h2;
} Key;

static void mix_bytes(Key *k, const void *p, size_t n)
{
    const unsigned char *b = p;
    for (size_t i = 0; i < n; i++) {
        k->h1 = (k->h1 ^ b[i]) * 0x100000001b3ull;
        k->h2 = (k->h2 + b[i] + 0x9E3779B97F4A7C15ull) * 0xff51afd7ed558ccdull;
        k->h2 ^= k->h2 >> 29;
    }
}

static void mix_program(Key *k, const Program *p)
{
    /* an instruction as one word: two multiplies each (a batch keys thousands of programs) */
    for (size_t i = 0; i < p->len; i++) {
        uint64_t w = p->code[i].addr << 1 | p->code[i].op;
        k->h1 = (k->h1 ^ w) * 0x100000001b3ull;
        k->h2 = (k->h2 + w + 0x9E3779B97F4A7C15ull) * 0xff51afd7ed558ccdull;
        k->h2 ^= k->h2 >> 29;
    }
    mix_bytes(k, &p->len, sizeof p->len);
    mix_bytes(k, &p->ncells, sizeof p->ncells);
    mix_bytes(k, p->inputs, p->ninputs * sizeof *p->inputs);
    mix_bytes(k, &p->ninputs, sizeof p->ninputs);
    mix_bytes(k, p->outputs, p->noutputs * sizeof *p->outputs);
    mix_bytes(k, &p->noutputs, sizeof p->noutputs);
}

static void enum_key(const TcGenEnum *g, uint64_t *k1, uint64_t *k2)
{
    Key k = {0xcbf29ce484222325ull, 0x6a09e667f3bcc909ull};
    int head[5] = {g->mode, (int)g->ticks, g->block, g->no_map, g->step_bits};
    mix_bytes(&k, head, sizeof head);
    mix_program(&k, g->a);
    if (g->b) {
        mix_program(&k, g->b);
        mix_bytes(&k, g->b_inputs, g->a->ninputs * sizeof *g->b_inputs);
        mix_bytes(&k, g->out_map, g->a->noutputs * sizeof *g->out_map);
    }
    if (g->spec) {
        const TcSpec *s = g->spec;
        mix_bytes(&k, &s->width, sizeof s->width);
        mix_bytes(&k, s->out, (size_t)s->width * sizeof s->out[0]);
        mix_bytes(&k, &s->nvars, sizeof s->nvars);
        mix_bytes(&k, s->var_bits, (size_t)s->nvars * sizeof s->var_bits[0]);
        for (int v = 0; v < s->nvars; v++)
            mix_bytes(&k, s->var_pos[v], (size_t)s->var_bits[v] * sizeof s->var_pos[v][0]);
        mix_bytes(&k, &s->nrpn, sizeof s->nrpn);
        for (int i = 0; i < s->nrpn; i++) {
            mix_bytes(&k, &s->rpn[i].op, sizeof s->rpn[i].op);
            mix_bytes(&k, &s->rpn[i].v, sizeof s->rpn[i].v);
        }
    }
    mix_bytes(&k, &g->target, sizeof g->target);
    *k1 = k.h1;
    *k2 = k.h2;
}

typedef struct {
    uint64_t k1, k2;
    TcModule m;
} EnumEntry;

static EnumEntry *enum_cache;
static size_t nenum, capenum;

static int lookup_enum(uint64_t k1, uint64_t k2, TcModule *m)
{
    int hit = 0;
    pthread_mutex_lock(&engine_lock);
    for (size_t i = 0; i < nenum; i++)
        if (enum_cache[i].k1 == k1 && enum_cache[i].k2 == k2) {
            *m = enum_cache[i].m;
            m->info.cached = 1;
            hit = 1;
            break;
        }
    pthread_mutex_unlock(&engine_lock);
    return hit;
}

static void remember_enum(uint64_t k1, uint64_t k2, const TcModule *m)
{
    pthread_mutex_lock(&engine_lock);
    if (nenum == capenum) {
        capenum = capenum ? 2 * capenum : 64;
        enum_cache = tc_xrealloc(enum_cache, capenum * sizeof *enum_cache);
    }
    enum_cache[nenum].k1 = k1;
    enum_cache[nenum].k2 = k2;
    enum_cache[nenum].m = *m;
    nenum++;
    pthread_mutex_unlock(&engine_lock);
}

char *tc_codegen_enum_for(const Enum *e, size_t *len, char *err, size_t errlen)
{
    EnumPlan pl;
    if (!plan_enum(e, &pl, err, errlen))
        return NULL;
    char *src = tc_codegen_enum(&pl.g, len);
    plan_free(&pl);
    return src;
}

/* The PTX module of n jobs as a quick-start build writes it (for inspection and ptxas tests) */
char *tc_codegen_ptx_for(const Enum *const *e, int n, const char *target, size_t *len, char *err,
                         size_t errlen)
{
    if (n < 1 || n > TC_MAX_KERNELS) {
        tc_fail(err, errlen, "a module of %d jobs: 1 to %d", n, TC_MAX_KERNELS);
        return NULL;
    }
    EnumPlan pl[TC_MAX_KERNELS];
    TcGenEnum *g[TC_MAX_KERNELS];
    int np = 0, ok = 1;
    for (int i = 0; ok && i < n; i++) {
        ok = plan_enum(e[i], &pl[i], err, errlen);
        if (ok) {
            g[np++] = &pl[i].g;
            if (!tc_ptx_enum_ok(g[i]))
                ok = tc_fail(err, errlen,
                             "the PTX writer takes equivalence and search jobs of one tick");
        }
    }
    char *src = ok ? tc_ptx_enum(g, n, target, NULL, len) : NULL;
    for (int i = 0; i < np; i++)
        plan_free(&pl[i]);
    return src;
}

/* ---- the autotuner's choices ---------------------------------------------------------------

   cuda_enum_tune measures kernels of one job that differ in threads per block and stretch length
   and keeps the fastest here, keyed by the job's default plan; every later launch of the same job
   (cuda_enum_run, the serving and batch paths, cuda_enum_run_static) takes the kernel of the
   choice. */
typedef struct {
    uint64_t k1, k2;
    int      block, step_bits;
} Tuned;

static Tuned tuned[256];
static size_t ntuned;

/* The tuned block and stretch for the job planned in g (default block, stretch of the cost
   model), when the autotuner has chosen them. */
static void apply_tuning(TcGenEnum *g)
{
    uint64_t k1, k2;
    enum_key(g, &k1, &k2);
    pthread_mutex_lock(&engine_lock);
    for (size_t i = 0; i < ntuned; i++)
        if (tuned[i].k1 == k1 && tuned[i].k2 == k2) {
            g->block = tuned[i].block;
            g->step_bits = tuned[i].step_bits;
            break;
        }
    pthread_mutex_unlock(&engine_lock);
}

static void remember_tuning(uint64_t k1, uint64_t k2, int block, int step_bits)
{
    pthread_mutex_lock(&engine_lock);
    size_t i = 0;
    while (i < ntuned && !(tuned[i].k1 == k1 && tuned[i].k2 == k2))
        i++;
    if (i == ntuned && ntuned < sizeof tuned / sizeof tuned[0])
        ntuned++;
    if (i < ntuned)
        tuned[i] = (Tuned){k1, k2, block, step_bits};
    pthread_mutex_unlock(&engine_lock);
}

/* Kernels compiled for a quick start (the serving loop's and a batch's compiled jobs): ptxas
   without optimisation.  Measured on GB300 over 90 batch and served jobs: NVRTC 0.053 s +
   8.3 us per NAND/STO instruction against 0.054 s + 13.9 us at -O2 (0.06 against 0.17 s for the
   heaviest batch jobs), the kernels running at about half the speed (1.7e15 against 3.5e15
   lane-ops/s), which a job that replaces interpreter time barely notices.  The source records
   the option, so the two builds are cached apart. */
#define FAST_NVRTC_OPT "--ptxas-options=-O0"

int tc_enum_ptx = 1;
int tc_enum_ptx_opt = 0;

int tc_enum_quick_ptx(const Enum *e)
{
    return tc_enum_ptx && (e->mode == EN_EQUIV || e->mode == EN_SEARCH) && e->ticks == 1 &&
           e->a && e->a->ninputs >= 1 && e->a->ninputs <= 64;
}

/* Build modes (the `fast` argument of the build and lookup functions):
     TC_BUILD_OPT      NVRTC with ptxas -O2, the kernel cuda_enum_run keeps;
     TC_BUILD_QUICK    a quick start: PTX written directly (ptxas at tc_enum_ptx_opt) for the jobs
                       the PTX writer takes, NVRTC with FAST_NVRTC_OPT for the rest; an optimised
                       build in the cache is taken instead (a batch's compiled jobs);
     TC_BUILD_QUICK_ONLY  the same, but never the optimised build (tests of quick builds);
     TC_BUILD_SERVE    PTX written directly with ptxas -O3 for the jobs the PTX writer takes (the
                       optimised build's speed at a third of NVRTC's compile time), the optimised
                       NVRTC build for the rest (a served stream's compiled jobs). */
static int is_quick(const TcGenEnum *g, int fast)
{
    return fast == TC_BUILD_QUICK || fast == TC_BUILD_QUICK_ONLY ||
           (fast == TC_BUILD_SERVE && tc_enum_ptx && tc_ptx_enum_ok(g));
}

static int ptx_opt(int fast)
{
    return fast == TC_BUILD_SERVE ? 3 : tc_enum_ptx_opt ? 3 : 0;
}

/* A quick build's key from the optimised build's: NVRTC's and the PTX writer's builds, and the
   latter at each ptxas level, are cached apart (they give the same results, but a test or a
   measurement may want the one it asked for) */
static void fast_key(const TcGenEnum *g, int fast, uint64_t *k2)
{
    *k2 ^= tc_enum_ptx && tc_ptx_enum_ok(g)
               ? 0xC2B2AE3D27D4EB4Full + (uint64_t)ptx_opt(fast)
               : 0x9E3779B97F4A7C15ull;
}

/* The cached kernel of plan g (keys k1, k2 of its optimised build) for build mode `fast`: the
   optimised NVRTC build, else for a quick mode the PTX writer's -O3 build, else the mode's own
   quick build (TC_BUILD_QUICK_ONLY: only its own) */
static int lookup_built(const TcGenEnum *g, int fast, uint64_t k1, uint64_t k2, TcModule *m)
{
    if (fast != TC_BUILD_QUICK_ONLY && lookup_enum(k1, k2, m))
        return 1;
    if (!is_quick(g, fast))
        return 0;
    uint64_t q = k2;
    if (fast == TC_BUILD_QUICK && tc_enum_ptx && tc_ptx_enum_ok(g)) {
        fast_key(g, TC_BUILD_SERVE, &q);
        if (lookup_enum(k1, q, m))
            return 1;
        q = k2;
    }
    fast_key(g, fast, &q);
    return lookup_enum(k1, q, m);
}

/* The loaded kernel of an enumeration, only when an earlier run of the same job compiled and
   loaded it (the optimised build, or the quick build of mode `fast`): no code generation, no
   compilation, no module load.  For cuda_enum_run_static, whose callers cannot allocate, and the
   serving loop's routing. */
int tc_enum_cached(const Enum *e, int fast, TcModule *m, char *err, size_t errlen)
{
    /* the maps in fixed buffers: this lookup allocates nothing */
    int in_map[EN_MAX_IN + 1], out_map[TC_CACHED_MAX_OUTPUTS + 1];
    uint32_t b_in[EN_MAX_IN + 1];
    if (!e || !e->a)
        return tc_fail(err, errlen, "no program");
    if (e->a->noutputs > TC_CACHED_MAX_OUTPUTS)
        return tc_fail(err, errlen, "cuda_enum_run_static: %zu outputs; at most %d here",
                       e->a->noutputs, TC_CACHED_MAX_OUTPUTS);
    EnumPlan pl;
    memset(&pl, 0, sizeof pl);
    pl.in_map = in_map;
    pl.out_map = out_map;
    pl.b_in = b_in;
    if (!plan_fill(e, &pl, err, errlen))
        return 0;
    apply_tuning(&pl.g);
    uint64_t k1, k2;
    enum_key(&pl.g, &k1, &k2);
    if (lookup_built(&pl.g, fast, k1, k2, m))
        return 1;
    return tc_fail(err, errlen, "cuda_enum_run_static: this job's kernel is not loaded; run the "
                   "same job once through cuda_enum_run first");
}

void tc_free(void *p)
{
    free(p);
}

/* ---- one enumeration in steps ---------------------------------------------------------------- */

/* Workspace of a launch: the hit counter, then 16 hits per warp, then a count per warp. */
#define WS_LIST 256u

/* Generated kernels compiled together into one module and not yet loaded: one kernel per job of
   a group (up to TC_MAX_KERNELS), so the group pays NVRTC's fixed cost once and loads once (a
   load waits for the device's running work).  Shared by the group's jobs until the last is
   loaded or dropped. */
struct TcEnumPending {
    char     *src;
    size_t    len;
    TcBuilt   b;
    int       n, refs, loaded;
    TcModule  m;  /* once loaded: kernel k in fn[k] */
    struct {
        uint64_t  k1, k2;
        TcGenWork work;
        int       block;
    } k[TC_MAX_KERNELS];
};

static void enum_pending_release(TcEnumPending *p)
{
    if (p && --p->refs == 0) {
        tc_built_free(&p->b);
        free(p->src);
        free(p);
    }
}

/* The module source of n jobs' kernels: one job's source as it is (kernel tc_enum); several,
   each in a namespace of its own with its kernel renamed tc_enum_<k> and its macros undefined
   after it (the common ones are defined alike by every job). */
static char *group_source(char **srcs, const size_t *lens, int n, size_t *len)
{
    if (n == 1) {
        char *s = tc_xmalloc(lens[0] + 1);
        memcpy(s, srcs[0], lens[0] + 1);
        *len = lens[0];
        return s;
    }
    static const char sig[] = ") tc_enum(const TcEnumArgs";
    size_t cap = 256, at = 0;
    for (int k = 0; k < n; k++)
        cap += lens[k] + 1024;
    char *o = tc_xmalloc(cap);
    for (int k = 0; k < n; k++) {
        at += (size_t)snprintf(o + at, cap - at, "namespace tcj%d {\n", k);
        const char *s = srcs[k], *hit = strstr(s, sig);
        size_t pre = hit ? (size_t)(hit - s) : lens[k];
        memcpy(o + at, s, pre);
        at += pre;
        if (hit) {
            at += (size_t)snprintf(o + at, cap - at, ") tc_enum_%d(const TcEnumArgs", k);
            size_t rest = lens[k] - pre - (sizeof sig - 1);
            memcpy(o + at, hit + sizeof sig - 1, rest);
            at += rest;
        }
        at += (size_t)snprintf(o + at, cap - at, "\n}\n");
        /* #undef every macro the job defined */
        for (const char *d = strstr(s, "#define "); d; d = strstr(d + 8, "#define ")) {
            const char *nm = d + 8, *e = nm;
            while ((*e >= 'A' && *e <= 'Z') || (*e >= 'a' && *e <= 'z') || (*e >= '0' && *e <= '9') ||
                   *e == '_')
                e++;
            if (at + (size_t)(e - nm) + 16 > cap) {
                cap = 2 * cap + (size_t)(e - nm) + 16;
                o = tc_xrealloc(o, cap);
            }
            at += (size_t)snprintf(o + at, cap - at, "#undef %.*s\n", (int)(e - nm), nm);
        }
    }
    o[at] = '\0';
    *len = at;
    return o;
}

/* The kernels for the plans in g[0..n): from the cache (m[i] filled, pend[i] NULL), else
   generated and compiled together (pend[i]: the group's build, for enum_module_load) in the build
   mode `fast` (TC_BUILD_*).  The jobs of a call that need building form at most two groups: one
   NVRTC program and one PTX module. */
static int enum_modules_build(TcGenEnum *const *g, int n, int fast, TcModule *m,
                              TcEnumPending **pend, int *kidx, char *err, size_t errlen)
{
    TcEnumPending *p[2] = {NULL, NULL};  /* [0] NVRTC, [1] PTX */
    TcGenEnum *gk[2][TC_MAX_KERNELS];
    int who[2][TC_MAX_KERNELS], nb[2] = {0, 0};
    for (int i = 0; i < n; i++) {
        pend[i] = NULL;
        kidx[i] = 0;
        uint64_t k1, k2;
        enum_key(g[i], &k1, &k2);
        if (lookup_built(g[i], fast, k1, k2, &m[i]))
            continue;
        const int quick = is_quick(g[i], fast);
        if (quick)
            fast_key(g[i], fast, &k2);
        const int kind = quick && tc_enum_ptx && tc_ptx_enum_ok(g[i]);
        /* PTX kernels run in blocks of 128: ptxas without optimisation takes more registers,
           and smaller blocks fill an SM's register file in finer steps */
        if (kind)
            g[i]->block = TC_PTX_BLOCK;
        if (!p[kind])
            p[kind] = tc_xcalloc(1, sizeof *p[kind]);
        int k = nb[kind]++;
        p[kind]->k[k].k1 = k1;
        p[kind]->k[k].k2 = k2;
        p[kind]->k[k].block = g[i]->block;
        gk[kind][k] = g[i];
        who[kind][k] = i;
        kidx[i] = k;
    }
    int ok = 1;
    if (p[0]) {
        char *srcs[TC_MAX_KERNELS];
        size_t lens[TC_MAX_KERNELS];
        for (int k = 0; k < nb[0]; k++) {
            gk[0][k]->work = &p[0]->k[k].work;
            srcs[k] = tc_codegen_enum(gk[0][k], &lens[k]);
            gk[0][k]->work = NULL;
            if (is_quick(gk[0][k], fast)) {
                static const char mark[] = "// built with " FAST_NVRTC_OPT "\n";
                char *s2 = tc_xmalloc(lens[k] + sizeof mark);
                memcpy(s2, mark, sizeof mark - 1);
                memcpy(s2 + sizeof mark - 1, srcs[k], lens[k] + 1);
                free(srcs[k]);
                srcs[k] = s2;
                lens[k] += sizeof mark - 1;
            }
        }
        p[0]->n = nb[0];
        p[0]->src = group_source(srcs, lens, nb[0], &p[0]->len);
        for (int k = 0; k < nb[0]; k++)
            free(srcs[k]);
        /* NVRTC's jobs of a call are all quick or all optimised (TC_BUILD_SERVE sends the quick
           ones to PTX) */
        ok = tc_module_build(p[0]->src, p[0]->len, is_quick(gk[0][0], fast) ? FAST_NVRTC_OPT : NULL,
                             &p[0]->b, err, errlen);
    }
    if (ok && p[1]) {
        char target[16];
        TcGenWork work[TC_MAX_KERNELS];
        snprintf(target, sizeof target, "sm_%d%da", tc_engine.cc_major, tc_engine.cc_minor);
        p[1]->n = nb[1];
        char *ptx = tc_ptx_enum(gk[1], nb[1], target, work, &p[1]->len);
        /* the text is the module cache's key: it records the optimisation level */
        p[1]->src = tc_xmalloc(p[1]->len + 32);
        p[1]->len = (size_t)sprintf(p[1]->src, "// ptxas -O%d\n%s", ptx_opt(fast), ptx);
        free(ptx);
        for (int k = 0; k < nb[1]; k++)
            p[1]->k[k].work = work[k];
        ok = tc_module_build_ptx(p[1]->src, p[1]->len, ptx_opt(fast), &p[1]->b, err, errlen);
    }
    for (int kind = 0; kind < 2; kind++) {
        if (!p[kind])
            continue;
        if (!ok) {
            tc_built_free(&p[kind]->b);
            free(p[kind]->src);
            free(p[kind]);
            continue;
        }
        p[kind]->refs = nb[kind];
        for (int k = 0; k < nb[kind]; k++)
            pend[who[kind][k]] = p[kind];
    }
    return ok;
}

/* Job i's kernel of a built group, loading the group's module first if no job of it has (the
   load waits for the device's running work); releases the job's share of the group. */
static int enum_module_load(TcEnumPending *p, int i, TcModule *m, char *err, size_t errlen)
{
    int ok = 1;
    if (!p->loaded) {
        char names[TC_MAX_KERNELS][24];
        const char *ptrs[TC_MAX_KERNELS];
        for (int k = 0; k < p->n; k++) {
            if (p->n == 1)
                snprintf(names[k], sizeof names[k], "tc_enum");
            else
                snprintf(names[k], sizeof names[k], "tc_enum_%d", k);
            ptrs[k] = names[k];
        }
        ok = tc_module_load(p->src, p->len, &p->b, ptrs, p->n, &p->m, err, errlen);
        if (ok) {
            p->loaded = 1;
            for (int k = 0; k < p->n; k++) {
                TcModule mk = p->m;
                mk.fn[0] = p->m.fn[k];
                mk.info.luts_per_step = p->k[k].work.luts_per_step;
                mk.info.luts_per_stretch = p->k[k].work.luts_per_stretch;
                mk.info.stretch_steps = p->k[k].work.stretch_steps;
                mk.info.compare_ops = p->k[k].work.compare_ops;
                mk.info.block = p->k[k].block;
                remember_enum(p->k[k].k1, p->k[k].k2, &mk);
            }
        }
    }
    if (ok) {
        *m = p->m;
        m->fn[0] = p->m.fn[i];
        struct cudaFuncAttributes fa;
        if (i > 0 && cudaFuncGetAttributes(&fa, (const void *)m->fn[0]) == cudaSuccess) {
            m->info.regs = fa.numRegs;
            m->info.local_bytes = (int)fa.localSizeBytes;
        }
        m->info.luts_per_step = p->k[i].work.luts_per_step;
        m->info.luts_per_stretch = p->k[i].work.luts_per_stretch;
        m->info.stretch_steps = p->k[i].work.stretch_steps;
        m->info.compare_ops = p->k[i].work.compare_ops;
        m->info.block = p->k[i].block;
    }
    enum_pending_release(p);
    return ok;
}

static int enum_module(TcGenEnum *g, int fast, TcModule *m, char *err, size_t errlen)
{
    TcEnumPending *p;
    int k;
    return enum_modules_build(&g, 1, fast, m, &p, &k, err, errlen) &&
           (!p || enum_module_load(p, 0, m, err, errlen));
}

/* The launch shape of job e on module m: as many blocks as are resident on the device at once
   (at most one warp per 32 words), each warp a contiguous run of the selected words. */
static int enum_shape(const Enum *e, TcEnumJob *j, char *err, size_t errlen)
{
    const int block = j->m.info.block;
    uint64_t space = 1ull << e->a->ninputs, sel, tried, pruns;
    tc_enum_shares(e, space, &sel, &tried, &pruns);
    j->base.space = space;
    j->base.tried = tried;
    j->base.ops = pruns * 512 * e->ticks * (e->a->len + (e->mode == EN_EQUIV ? e->b->len : 0));
    int per_sm = 0;
    if (!tc_cu_check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                         &per_sm, (const void *)j->m.fn[0], block, 0),
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
    uint64_t per_warp = (words + warps - 1) / warps;
    per_warp = (per_warp + 31) / 32 * 32;
    if (!per_warp)
        per_warp = 32;
    j->blocks = blocks;
    j->warps = warps;
    j->words = words;
    j->space = space;
    j->per_warp = per_warp;
    j->parts = (uint32_t)e->parts;
    j->part = (uint32_t)e->part;
    j->nsel = (uint32_t)(e->part_end - e->part + 1);
    return 1;
}

int tc_enum_jobs_build(const Enum *const *e, TcEnumJob *const *j, int n, int fast, char *err,
                       size_t errlen)
{
    if (n < 1 || n > TC_MAX_KERNELS)
        return tc_fail(err, errlen, "a build of %d jobs: 1 to %d", n, TC_MAX_KERNELS);
    EnumPlan pl[TC_MAX_KERNELS];
    TcGenEnum *g[TC_MAX_KERNELS];
    TcModule m[TC_MAX_KERNELS];
    TcEnumPending *pend[TC_MAX_KERNELS];
    int kidx[TC_MAX_KERNELS];
    int np = 0, ok = 1;
    /* the refusals first (no device needed for them), then the device */
    for (int i = 0; ok && i < n; i++) {
        memset(j[i], 0, sizeof *j[i]);
        ok = plan_enum(e[i], &pl[i], err, errlen);
        if (ok) {
            np++;
            g[i] = &pl[i].g;
        }
    }
    if (ok)
        ok = cuda_engine_init(0, err, errlen);
    for (int i = 0; ok && i < n; i++)
        apply_tuning(&pl[i].g);
    if (ok)
        ok = enum_modules_build(g, n, fast, m, pend, kidx, err, errlen);
    for (int i = 0; ok && i < n; i++) {
        j[i]->m = m[i];
        j[i]->pending = pend[i];
        j[i]->pidx = kidx[i];
    }
    for (int i = 0; i < np; i++)
        plan_free(&pl[i]);
    return ok;
}

int tc_enum_job_build(const Enum *e, TcEnumJob *j, int fast, char *err, size_t errlen)
{
    return tc_enum_jobs_build(&e, &j, 1, fast, err, errlen);
}

int tc_enum_job_load(const Enum *e, TcEnumJob *j, char *err, size_t errlen)
{
    if (j->pending) {
        TcEnumPending *p = j->pending;
        j->pending = NULL;
        if (!enum_module_load(p, j->pidx, &j->m, err, errlen))
            return 0;
    }
    return enum_shape(e, j, err, errlen);
}

void tc_enum_job_drop(TcEnumJob *j)
{
    enum_pending_release(j->pending);
    j->pending = NULL;
}

int tc_enum_job_prepare(const Enum *e, TcEnumJob *j, int fast, char *err, size_t errlen)
{
    if (!tc_enum_job_build(e, j, fast, err, errlen))
        return 0;
    if (!tc_enum_job_load(e, j, err, errlen)) {
        tc_enum_job_drop(j);
        return 0;
    }
    return 1;
}

size_t tc_enum_job_ws_bytes(const TcEnumJob *j)
{
    return WS_LIST + (size_t)j->warps * (16 * 8 + 4);
}

size_t tc_enum_job_ws_max(void)
{
    /* at most 2,048 threads per SM: 64 warps */
    return WS_LIST + (size_t)tc_engine.sms * 64 * (16 * 8 + 4);
}

static int launch_enum(const TcEnumJob *j, void *hits, void *list, void *count, cudaStream_t st,
                       char *err, size_t errlen)
{
    TcEnumArgs args;
    memset(&args, 0, sizeof args);
    args.words = j->words;
    args.space = j->space;
    args.per_warp = j->per_warp;
    args.parts = j->parts;
    args.part = j->part;
    args.nsel = j->nsel;
    args.hits = hits;
    args.list = list;
    args.count = count;
    void *params[] = {&args};
    return tc_cu_check(cudaMemsetAsync(hits, 0, 8, st), "memset", err, errlen) &&
           tc_cu_check(cudaLaunchKernel((const void *)j->m.fn[0], dim3u((unsigned)j->blocks),
                                        dim3u((unsigned)j->m.info.block), params, 0, st),
                       "launch tc_enum", err, errlen);
}

int tc_enum_job_launch(const TcEnumJob *j, void *dev_ws, void *host_ws, cudaStream_t st, char *err,
                       size_t errlen)
{
    char *d = dev_ws;
    return launch_enum(j, d, d + WS_LIST, d + WS_LIST + (size_t)j->warps * 16 * 8, st, err,
                       errlen) &&
           tc_cu_check(cudaMemcpyAsync(host_ws, dev_ws, tc_enum_job_ws_bytes(j),
                                       cudaMemcpyDeviceToHost, st),
                       "workspace copy", err, errlen);
}

void tc_enum_job_result(const TcEnumJob *j, const void *host_ws, EnumResult *r)
{
    const char *h = host_ws;
    const uint64_t *list = (const uint64_t *)(h + WS_LIST);
    const uint32_t *count = (const uint32_t *)(h + WS_LIST + (size_t)j->warps * 16 * 8);
    *r = j->base;
    memcpy(&r->hits, h, 8);
    r->threads = (int)(j->blocks * (uint64_t)j->m.info.block);
    /* every warp's list: a kernel whose enumeration order is permuted does not find the
       smallest hits in the first warps */
    for (uint64_t w = 0; w < j->warps && r->hits; w++)
        for (uint32_t i = 0; i < count[w]; i++)
            cuda_enum_add_hit(r, list[w * 16 + i]);
}

/* Runs a prepared job on the engine's stream into the engine's workspace; r gets its result. */
static int run_prepared(const TcEnumJob *jp, EnumResult *r, char *err, size_t errlen)
{
    const TcEnumJob j = *jp;
    uint64_t warps = j.warps;
    if (!tc_scratch(&tc_engine.ws_hits, 8, err, errlen) ||
        !tc_scratch(&tc_engine.ws_list, warps * 16 * 8, err, errlen) ||
        !tc_scratch(&tc_engine.ws_count, warps * 4, err, errlen))
        return 0;
    cudaStream_t st = tc_engine.stream;
    if (!tc_cu_check(cudaEventRecord(tc_engine.ev0, st), "event", err, errlen) ||
        !launch_enum(&j, tc_engine.ws_hits.ptr, tc_engine.ws_list.ptr, tc_engine.ws_count.ptr, st,
                     err, errlen) ||
        !tc_cu_check(cudaEventRecord(tc_engine.ev1, st), "event", err, errlen))
        return 0;
    *r = j.base;
    uint64_t hits = 0;
    uint32_t *count = tc_xmalloc(warps * 4);
    cudaError_t rc = cudaMemcpyAsync(&hits, tc_engine.ws_hits.ptr, 8, cudaMemcpyDeviceToHost, st);
    if (rc == cudaSuccess)
        rc = cudaMemcpyAsync(count, tc_engine.ws_count.ptr, warps * 4, cudaMemcpyDeviceToHost, st);
    if (rc == cudaSuccess)
        rc = cudaStreamSynchronize(st);
    if (rc != cudaSuccess) {
        free(count);
        return tc_cu_check(rc, "tc_enum", err, errlen);
    }
    /* every warp's list (a kernel whose enumeration order is permuted does not find the
       smallest hits in the first warps), in one copy when there are hits */
    if (hits) {
        uint64_t *list = tc_xmalloc(warps * 16 * 8);
        rc = cudaMemcpy(list, tc_engine.ws_list.ptr, warps * 16 * 8, cudaMemcpyDeviceToHost);
        if (rc != cudaSuccess) {
            free(list);
            free(count);
            return tc_cu_check(rc, "hits", err, errlen);
        }
        for (uint64_t w = 0; w < warps; w++)
            for (uint32_t i = 0; i < count[w]; i++)
                cuda_enum_add_hit(r, list[w * 16 + i]);
        free(list);
    }
    free(count);
    float ms = 0;
    cudaEventElapsedTime(&ms, tc_engine.ev0, tc_engine.ev1);
    r->seconds = ms / 1e3;
    r->hits = hits;
    r->threads = (int)(j.blocks * (uint64_t)j.m.info.block);
    tc_engine.last = j.m.info;
    tc_engine.last_kernel_ms = ms;
    tc_engine.last_grid = (unsigned)j.blocks;
    tc_engine.last_block = (unsigned)j.m.info.block;
    return 1;
}

/* cuda_enum_run's build mode (TC_BUILD_*; tests and measurements of the other builds) */
int tc_enum_run_fast = 0;

int cuda_enum_run(const Enum *e, EnumResult *r, char *err, size_t errlen)
{
    memset(r, 0, sizeof *r);
    TcEnumJob j;
    return tc_enum_job_prepare(e, &j, tc_enum_run_fast, err, errlen) &&
           run_prepared(&j, r, err, errlen);
}

/* ---- the autotuner --------------------------------------------------------------------------- */

typedef struct {
    const Enum *e;
    TcGenEnum   g;
    TcEnumJob   j;
    int         ok;
    char        err[256];
} Candidate;

static void *compile_candidate(void *arg)
{
    Candidate *c = arg;
    memset(&c->j, 0, sizeof c->j);
    c->ok = enum_module(&c->g, 0, &c->j.m, c->err, sizeof c->err) &&
            enum_shape(c->e, &c->j, c->err, sizeof c->err);
    return NULL;
}

/* Kernels of job e for threads per block 128, 256 and 512 and, where the work splits into
   stretches, stretches of 8, 16 and 32 steps: compiled in parallel host threads, each run once on
   a probe -- the whole job, or the share of its chunks that takes about 20 ms -- with every
   result compared, then timed three times; the fastest becomes the job's kernel for every later
   launch.  t gets each candidate's best time. */
int cuda_enum_tune(const Enum *e, CudaTune *t, char *err, size_t errlen)
{
    memset(t, 0, sizeof *t);
    EnumPlan pl;
    if (!cuda_engine_init(0, err, errlen) || !plan_enum(e, &pl, err, errlen))
        return 0;
    uint64_t k1, k2;
    enum_key(&pl.g, &k1, &k2);  /* the default plan's key: the tuning table's */
    /* the probe: a share of about 20 ms at the generated code's rate (2e15 lane-ops/s) */
    double work = (double)(1ull << e->a->ninputs) * e->ticks *
                  (double)(e->a->len + (e->mode == EN_EQUIV ? e->b->len : 0)) *
                  (e->part_end - e->part + 1) / e->parts;
    uint64_t chunks = ((1ull << e->a->ninputs) + 32767) / 32768, parts = 1;
    while (work / parts > 2e15 * 0.02 && parts * 2 <= chunks)
        parts *= 2;
    Enum probe = *e;
    if (parts > 1) {
        probe.part = probe.part_end = 0;
        probe.parts = (int)parts;
    }
    t->probe_fraction = parts > 1 ? 1.0 / (double)parts : 1.0;
    static const int blocks[3] = {128, 256, 512};
    int splits = pl.g.ticks == 1 && !pl.g.no_map && e->a->ninputs >= 13;
    Candidate c[9];
    pthread_t tid[9];
    int n = 0;
    for (int b = 0; b < 3; b++)
        for (int sb = splits ? 3 : 0; sb <= (splits ? 5 : 0); sb++) {
            c[n].e = parts > 1 ? &probe : e;
            c[n].g = pl.g;
            c[n].g.block = blocks[b];
            c[n].g.step_bits = sb;
            c[n].ok = 0;
            n++;
        }
    int started = 0;
    for (; started < n; started++)
        if (pthread_create(&tid[started], NULL, compile_candidate, &c[started]) != 0)
            break;
    for (int i = 0; i < started; i++)
        pthread_join(tid[i], NULL);
    int ok = 1, best = -1;
    EnumResult want;
    memset(&want, 0, sizeof want);
    for (int i = 0; i < n && ok; i++) {
        t->cand[i].block = c[i].g.block;
        t->cand[i].step_bits = c[i].g.step_bits;
        t->cand[i].ms = -1;
        if (i >= started || !c[i].ok)
            continue;  /* e.g. too many registers for 512 threads: not a candidate */
        EnumResult r;
        if (!run_prepared(&c[i].j, &r, err, errlen)) {
            ok = 0;
            break;
        }
        if (best < 0 && t->ncand == 0)
            want = r;
        if (r.hits != want.hits || r.nhit != want.nhit ||
            memcmp(r.hit, want.hit, sizeof r.hit) != 0) {
            ok = tc_fail(err, errlen, "autotune: candidate %d gives a different result", i);
            break;
        }
        double ms = 1e30;
        for (int rep = 0; rep < 3 && ok; rep++) {
            ok = run_prepared(&c[i].j, &r, err, errlen);
            if (ok && r.seconds * 1e3 < ms)
                ms = r.seconds * 1e3;
        }
        t->cand[i].ms = ms;
        t->ncand++;
        if (best < 0 || ms < t->cand[best].ms)
            best = i;
    }
    t->n = n;
    t->best = best;
    if (ok && best < 0)
        ok = tc_fail(err, errlen, "autotune: no candidate compiled: %s", c[0].err);
    if (ok)
        remember_tuning(k1, k2, c[best].g.block, c[best].g.step_bits);
    plan_free(&pl);
    return ok;
}

/* ---- truth tables --------------------------------------------------------------------------- */

int cuda_table(const Program *p, unsigned ticks, uint8_t *vals, char *err, size_t errlen)
{
    if (!p)
        return tc_fail(err, errlen, "no program");
    if (p->special)
        return tc_fail(err, errlen, "this program's machines read each other (id or link cells), "
                       "so they run as a cube: --table and --engine do not apply");
    if (p->ninputs == 0 || p->ninputs > 20)
        return tc_fail(err, errlen, "--table needs between 1 and 20 .in cells, this program has "
                       "%zu", p->ninputs);
    if (ticks < 1)
        return tc_fail(err, errlen, "--ticks must be at least 1");
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    size_t len;
    char *src = tc_codegen_table(p, ticks, TC_ENUM_BLOCK, &len);
    static const char *const names[] = {"tc_table"};
    TcModule m;
    int ok = tc_module(src, len, names, 1, NULL, &m, err, errlen);
    free(src);
    if (!ok)
        return 0;
    uint64_t rows = 1ull << p->ninputs, words = (rows + 31) / 32;
    size_t cols = p->noutputs ? p->noutputs : 1;
    size_t bytes = cols * words * 4;
    uint32_t *d = NULL, *h = tc_xmalloc(bytes);
    cudaStream_t st = tc_engine.stream;
    void *params[] = {&d, &words};
    ok = tc_cu_check(cudaMalloc((void **)&d, bytes), "cudaMalloc", err, errlen) &&
         tc_cu_check(cudaLaunchKernel((const void *)m.fn[0],
                                      dim3u((unsigned)((words + TC_ENUM_BLOCK - 1) / TC_ENUM_BLOCK)),
                                      dim3u(TC_ENUM_BLOCK), params, 0, st),
                     "launch tc_table", err, errlen) &&
         tc_cu_check(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, st), "table", err,
                     errlen) &&
         tc_cu_check(cudaStreamSynchronize(st), "tc_table", err, errlen);
    if (d)
        cudaFree(d);
    if (ok)
        for (uint64_t r = 0; r < rows; r++)
            for (size_t c = 0; c < cols; c++)
                vals[r * cols + c] = (uint8_t)((h[c * words + (r >> 5)] >> (r & 31)) & 1u);
    free(h);
    tc_engine.last = m.info;
    return ok;
}

/* The module source of n jobs built together (kernels tc_enum_0 ..), as the compile threads
   make it; for tests. */
char *tc_codegen_enum_group(const Enum *const *e, int n, size_t *len, char *err, size_t errlen)
{
    if (n < 1 || n > TC_MAX_KERNELS) {
        tc_fail(err, errlen, "a group of %d jobs: 1 to %d", n, TC_MAX_KERNELS);
        return NULL;
    }
    char *srcs[TC_MAX_KERNELS];
    size_t lens[TC_MAX_KERNELS];
    for (int i = 0; i < n; i++) {
        srcs[i] = tc_codegen_enum_for(e[i], &lens[i], err, errlen);
        if (!srcs[i]) {
            for (int k = 0; k < i; k++)
                free(srcs[k]);
            return NULL;
        }
    }
    char *out = group_source(srcs, lens, n, len);
    for (int i = 0; i < n; i++)
        free(srcs[i]);
    return out;
}
