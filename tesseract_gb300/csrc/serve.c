/* Serving with continuous batching: jobs arrive over time (an arrival time per job), are admitted
   by footprint as device memory and in-flight slots free up, and run on one of two engines,
   chosen per job when it arrives:

   - waves of the batched interpreter: the jobs admitted together run in one persistent kernel,
     on one of several streams, with a share of the GPU's blocks so that a newer wave starts
     while older ones still run.  A job is finished the moment its last work unit is (the kernel
     raises a flag in host-mapped memory), not when its wave ends;
   - the generated-kernel engine of cuda_enum_run, for jobs whose work is large enough that the
     GPU time compiled code saves outweighs their share of the compile threads: host threads
     generate and compile (NVRTC, cached by what the generator reads), and the main loop
     launches each compiled job on a stream of its own into a preallocated workspace.

   The host loop never blocks on the device: it admits, launches, polls the flags and events and
   frees.  A job's result does not depend on the engine, the wave or the mix: both engines
   compute the whole enumeration of that one job. */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "batch.h"
#include "engine.h"

typedef struct TcWave TcWave;
int    tc_wave_prepare(TcWave **out, const Enum *const *jobs, int njobs, char *err, size_t errlen);
int    tc_wave_launch(TcWave *w, cudaStream_t stream, double share, char *err, size_t errlen);
int    tc_wave_job_done(const TcWave *w, int i);
int    tc_wave_finished(const TcWave *w);
void   tc_wave_result(const TcWave *w, int i, EnumResult *r);
size_t tc_wave_bytes(const TcWave *w);
void   tc_wave_free(TcWave *w);
void   tc_wave_pool_trim(void);

#define MAX_STREAMS 8
#define MAX_COMPILED 8       /* compiled jobs on the device at once, one stream each */
#define MAX_THREADS 64

/* Rates for routing, measured on GB300, in NAND/STO lane-ops/s: the batched interpreter's and
   generated code's on random programs; NVRTC's time for a generated kernel as a constant plus a
   cost per NAND/STO instruction.  The interpreter reaches ~1.4e14 on the 4,096-job batch alone;
   in the served mix, in waves beside compiled jobs, half of 9e13 routes better (Poisson 2,000
   jobs/s, widths to 34: 114.9 against 111.5 jobs/s, p50 0.31 against 1.49 s, p99 2.47 against
   2.73 s; widths to 22 unchanged).  A served stream keeps the GPU busy, so its compiled jobs get
   the optimised build; NVRTC alone takes 0.054 s + 13.9 us per NAND/STO instruction on one host
   thread and the code runs at 3.5e15 (median, fitted over 90 batch and served jobs), but in the
   serving loop a compile thread also waits for its module load (a load synchronises the
   context, so it waits for the waves in flight), and the figures below, which include that
   wait, route better (widths to 34: 121 against 114 jobs/s).  A batch waits on its compiles,
   so its compiled jobs get the quick-start build (ptxas without optimisation): 0.053 s + 8.3 us
   per instruction, running at 1.7e15, and their loads wait until the interpreter has every
   job. */
#define RATE_INTERP 4.5e13
#define RATE_COMPILED 2.0e15
#define COMPILE_S0 0.1
#define COMPILE_S_PER_INSTR 4.0e-5
#define RATE_COMPILED_FAST 1.7e15
#define COMPILE_S0_FAST 0.053
#define COMPILE_S_PER_INSTR_FAST 8.3e-6
/* A batch's equivalence and search jobs are built from PTX written directly (ptxgen.c): measured
   on the GB300 over 78 jobs of the 4,096-job batch, 0.0153 s + 2.63 us per NAND/STO instruction
   (ptxas without optimisation through nvJitLink, against 0.051 s + 9.2 us through NVRTC), the
   kernels at about 1.1e15 lane-ops/s on the heavier jobs. */
#define RATE_COMPILED_PTX 1.1e15
/* A served stream's equivalence and search jobs are built from PTX with ptxas -O3: 0.020 s +
   6.6 us per instruction against NVRTC's 0.058 s + 13.3 us (same 78 jobs), the kernels as fast
   (3.4e15 lane-ops/s on the heavier jobs, both).  In the serving model's terms, which include a
   compile thread's wait for its module load: */
#define COMPILE_S0_SERVE_PTX 0.063
#define COMPILE_S_PER_INSTR_SERVE_PTX 3.3e-5
/* 1 (default): a served stream's equivalence and search jobs are built so; 0: by NVRTC */
int tc_serve_quick = 1;
#define COMPILE_S0_PTX 0.0153
#define COMPILE_S_PER_INSTR_PTX 2.63e-6
/* A job whose kernel is already compiled (the cache is keyed by what the code generator reads)
   costs only its launch and the polling of its event: about this many seconds. */
#define LAUNCH_S 3.0e-5

typedef struct {
    TcWave *w;
    int    *ids;      /* job numbers of the wave */
    int     n, left;  /* jobs, jobs not finished */
    size_t  bytes;
} Flight;

/* ---- the compile threads -------------------------------------------------------------------- */

typedef struct {
    pthread_mutex_t     mu;
    pthread_cond_t      cv;
    const Enum *const  *jobs;
    TcEnumJob          *prep;            /* per job */
    int                *queue, qhead, qtail;
    int                *ready, rhead, rtail;
    int                 stop, failed;
    char                err[512];
    int                 defer;            /* build only: the host loop loads (a batch) */
    int                 threads;
    double              busy;             /* host seconds spent building or preparing */
} Compiler;

/* Jobs a compile thread builds together (one NVRTC program, one module load): NVRTC's fixed
   cost (0.053 s of a heavy job's 0.14 s) is paid once, and a load waits for the device's running
   work once for the group. */
#define COMPILE_GROUP TC_MAX_KERNELS
int tc_compile_group = 4;  /* jobs a compile thread takes at most (1..COMPILE_GROUP) */

static void *compile_worker(void *arg)
{
    Compiler *c = arg;
    for (;;) {
        pthread_mutex_lock(&c->mu);
        while (c->qhead == c->qtail && !c->stop)
            pthread_cond_wait(&c->cv, &c->mu);
        if (c->qhead == c->qtail) {
            pthread_mutex_unlock(&c->mu);
            return NULL;
        }
        /* a fair share of the queue, up to COMPILE_GROUP jobs: the other threads get theirs */
        int waiting = c->qtail - c->qhead, n = 1;
        while (n < tc_compile_group && n < COMPILE_GROUP && n * c->threads < waiting)
            n++;
        int ids[COMPILE_GROUP];
        for (int i = 0; i < n; i++)
            ids[i] = c->queue[c->qhead++];
        pthread_mutex_unlock(&c->mu);
        char e2[512];
        const Enum *es[COMPILE_GROUP];
        TcEnumJob *js[COMPILE_GROUP];
        for (int i = 0; i < n; i++) {
            es[i] = c->jobs[ids[i]];
            js[i] = &c->prep[ids[i]];
        }
        double t0 = tc_now();
        int ok = tc_enum_jobs_build(es, js, n,
                                    c->defer ? TC_BUILD_QUICK
                                    : tc_serve_quick ? TC_BUILD_SERVE : TC_BUILD_OPT, e2, sizeof e2);
        for (int i = 0; ok && !c->defer && i < n; i++)
            if (!tc_enum_job_load(es[i], js[i], e2, sizeof e2)) {
                for (int k = i; k < n; k++)
                    tc_enum_job_drop(js[k]);
                ok = 0;
            }
        double dt = tc_now() - t0;
        pthread_mutex_lock(&c->mu);
        c->busy += dt;
        if (ok) {
            for (int i = 0; i < n; i++)
                c->ready[c->rtail++] = ids[i];
        } else if (!c->failed) {
            c->failed = 1;
            snprintf(c->err, sizeof c->err, "job %d: %s", ids[0], e2);
        }
        pthread_mutex_unlock(&c->mu);
    }
}

/* Hands held jobs to the compile threads. */
static void release_held(Compiler *c, const int *ids, int n)
{
    pthread_mutex_lock(&c->mu);
    for (int i = 0; i < n; i++)
        c->queue[c->qtail++] = ids[i];
    pthread_cond_broadcast(&c->cv);
    pthread_mutex_unlock(&c->mu);
}

typedef struct {
    int          id;          /* -1: free */
    cudaStream_t st;
    cudaEvent_t  done;
    void        *dev, *host;  /* workspace and its pinned host copy */
} Slot;

/* Compiled code for job e when the GPU time it saves over the interpreter (running at
   rate_interp) is worth more than its compile time spread over the compile threads -- or, when
   its kernel is in the cache already, more than a launch. */
static int route_compiled(const Enum *e, const CudaServeOpts *o, int threads, double rate_interp)
{
    if (o->route == CUDA_SERVE_INTERPRETER || threads < 1)
        return 0;
    if (o->route == CUDA_SERVE_COMPILED)
        return 1;
    double instrs = (double)e->a->len + (e->mode == EN_EQUIV ? (double)e->b->len : 0.0);
    double work = (double)(1ull << e->a->ninputs) * (double)e->ticks * instrs;
    TcModule m;
    char why[8];
    double saved = work / rate_interp - work / RATE_COMPILED;
    if (tc_serve_quick && tc_enum_quick_ptx(e)) {
        if (tc_enum_cached(e, TC_BUILD_SERVE, &m, why, sizeof why))
            return saved > LAUNCH_S;
        return saved > (COMPILE_S0_SERVE_PTX + COMPILE_S_PER_INSTR_SERVE_PTX * instrs) / threads;
    }
    if (tc_enum_cached(e, TC_BUILD_OPT, &m, why, sizeof why))
        return saved > LAUNCH_S;
    return saved > (COMPILE_S0 + COMPILE_S_PER_INSTR * instrs) / threads;
}

/* The routing model's figures for a batch planner (quick-start builds): seconds to compile a job
   of `instrs` NAND/STO instructions (0 when its kernel is cached), the GPU seconds of `work`
   lane-ops on generated code, and a launch's cost. */
double tc_route_compile_s(const Enum *e, double instrs)
{
    TcModule m;
    char why[8];
    if (tc_enum_cached(e, TC_BUILD_QUICK, &m, why, sizeof why))
        return 0.0;
    return tc_enum_quick_ptx(e) ? COMPILE_S0_PTX + COMPILE_S_PER_INSTR_PTX * instrs
                                : COMPILE_S0_FAST + COMPILE_S_PER_INSTR_FAST * instrs;
}

double tc_route_compiled_s(const Enum *e, double work)
{
    return work / (tc_enum_quick_ptx(e) ? RATE_COMPILED_PTX : RATE_COMPILED_FAST) + LAUNCH_S;
}

static void nap(void)
{
    struct timespec t = {0, 20000};  /* 20 us */
    nanosleep(&t, NULL);
}

/* The loop of cuda_serve_run, with the interpreter's routing rate as a parameter: in the served
   mix its waves share the GPU with compiled jobs and run at about RATE_INTERP; a batch's single
   wave (tc_serve_batch) has the GPU nearly to itself. */
static int serve(const Enum *const *jobs, const double *arrival, int njobs,
                 const CudaServeOpts *opts, double rate_interp, const signed char *route,
                 int first_wave, double *start, double *finish, EnumResult *results,
                 int *engine_used, char *err, size_t errlen);

/* when the last call's first interpreter wave went out, in seconds from its start (-1: none) */
double tc_serve_last_wave_at = -1;
/* the last run's jobs routed to generated code on arrival, those a batch's interpreter took
   back from the compile queue, and the compile threads' busy seconds */
int    tc_serve_last_routed, tc_serve_last_taken_back;
double tc_serve_last_compile_busy, tc_serve_last_compile_load, tc_serve_last_loop_end;

int cuda_serve_run(const Enum *const *jobs, const double *arrival, int njobs,
                   const CudaServeOpts *opts, double *start, double *finish, EnumResult *results,
                   int *engine_used, char *err, size_t errlen)
{
    return serve(jobs, arrival, njobs, opts, RATE_INTERP, NULL, 0, start, finish, results,
                 engine_used, err, errlen);
}

/* Every job arriving at once with its engine chosen by the caller (route[i]: 1 generated code,
   0 the interpreter). */
int tc_serve_batch(const Enum *const *jobs, int njobs, const CudaServeOpts *opts,
                   const signed char *route, int first_wave, double *finish, EnumResult *results,
                   int *engine_used, char *err, size_t errlen)
{
    double *zero = tc_xcalloc((size_t)njobs, sizeof *zero);
    double *start = tc_xcalloc((size_t)njobs, sizeof *start);
    int ok = serve(jobs, zero, njobs, opts, RATE_INTERP, route, first_wave, start, finish, results,
                   engine_used, err, errlen);
    free(zero);
    free(start);
    return ok;
}

static int serve(const Enum *const *jobs, const double *arrival, int njobs,
                 const CudaServeOpts *opts, double rate_interp, const signed char *route,
                 int first_wave, double *start, double *finish, EnumResult *results,
                 int *engine_used, char *err, size_t errlen)
{
    if (njobs <= 0)
        return 1;
    if (!cuda_engine_init(0, err, errlen))
        return 0;
    CudaServeOpts o = *opts;
    if (o.streams < 1)
        o.streams = 4;
    if (o.streams > MAX_STREAMS)
        o.streams = MAX_STREAMS;
    if (o.max_inflight_jobs < 1)
        o.max_inflight_jobs = 4096;
    if (o.max_device_bytes == 0)
        o.max_device_bytes = (size_t)8 << 30;
    if (o.max_wave_jobs < 1)
        o.max_wave_jobs = 1024;
    if (o.share <= 0 || o.share > 1)
        o.share = 0.5;
    int threads = o.compile_threads == 0 ? 12 : o.compile_threads;
    if (threads > MAX_THREADS)
        threads = MAX_THREADS;
    if (o.route == CUDA_SERVE_COMPILED && threads < 1)
        threads = 1;
    if (o.route == CUDA_SERVE_INTERPRETER)
        threads = 0;
    int nslots = threads > 0 ? (o.compiled_slots > 0 ? o.compiled_slots : 4) : 0;
    if (nslots > MAX_COMPILED)
        nslots = MAX_COMPILED;

    int ok = 1;
    cudaStream_t st[MAX_STREAMS];
    int busy[MAX_STREAMS];
    int nst = 0;
    for (; nst < o.streams; nst++) {
        busy[nst] = 0;
        if (!tc_cu_check(cudaStreamCreateWithFlags(&st[nst], cudaStreamNonBlocking), "stream",
                         err, errlen)) {
            ok = 0;
            break;
        }
    }
    /* compiled-job slots: the largest workspace any launch on this device can need */
    Slot slot[MAX_COMPILED];
    memset(slot, 0, sizeof slot);
    size_t ws_max = tc_enum_job_ws_max();
    int nsl = 0;
    for (; ok && nsl < nslots; nsl++) {
        slot[nsl].id = -1;
        ok = tc_cu_check(cudaStreamCreateWithFlags(&slot[nsl].st, cudaStreamNonBlocking),
                         "stream", err, errlen) &&
             tc_cu_check(cudaEventCreateWithFlags(&slot[nsl].done, cudaEventDisableTiming),
                         "event", err, errlen) &&
             tc_cu_check(cudaMalloc(&slot[nsl].dev, ws_max), "cudaMalloc", err, errlen) &&
             tc_cu_check(cudaHostAlloc(&slot[nsl].host, ws_max, cudaHostAllocDefault),
                         "cudaHostAlloc", err, errlen);
    }
    Compiler cc;
    memset(&cc, 0, sizeof cc);
    pthread_mutex_init(&cc.mu, NULL);
    pthread_cond_init(&cc.cv, NULL);
    cc.jobs = jobs;
    /* a batch's compile threads only build, for a quick start: loading a module waits for the
       device's running work (it synchronises the context), which would hold each compile thread
       for most of an interpreter wave; the host loop loads the builds once the interpreter has
       everything */
    cc.defer = route != NULL;
    cc.threads = threads > 0 ? threads : 1;
    cc.prep = tc_xcalloc((size_t)njobs, sizeof *cc.prep);
    cc.queue = tc_xmalloc((size_t)njobs * sizeof *cc.queue);
    cc.ready = tc_xmalloc((size_t)njobs * sizeof *cc.ready);
    pthread_t tid[MAX_THREADS];
    int nthreads = 0;
    for (; ok && nthreads < threads; nthreads++)
        if (pthread_create(&tid[nthreads], NULL, compile_worker, &cc) != 0)
            break;

    Flight fl[MAX_STREAMS];
    memset(fl, 0, sizeof fl);
    int next = 0, finished = 0, inflight = 0;
    size_t bytes = 0;
    int *ready = tc_xmalloc((size_t)njobs * sizeof *ready), nready = 0, rhead = 0;
    const Enum **wj = tc_xmalloc((size_t)njobs * sizeof *wj);
    /* a batch holds its compiles until its first interpreter wave is out: packing the wave
       needs the host's cores first */
    int held = route != NULL, nheld = 0;
    int *held_ids = tc_xmalloc((size_t)njobs * sizeof *held_ids);
    int *loaded = tc_xmalloc((size_t)njobs * sizeof *loaded), nloaded = 0, lhead = 0;
    TcWave *pending = NULL;  /* a wave prepared but not yet admitted */
    int pending_n = 0;
    size_t pending_need = 0;
    double t0 = tc_now(), wave_launched_at = -1, load_s = 0;
    int routed = 0, taken_back = 0, loads_open = !cc.defer;
    while (ok && finished < njobs) {
        double now = tc_now() - t0;
        int progress = 0;
        /* arrivals: to the interpreter's queue or the compile threads */
        while (next < njobs && arrival[next] <= now) {
            int compiled = route ? route[next] && nthreads > 0
                                 : route_compiled(jobs[next], &o, nthreads, rate_interp);
            if (engine_used)
                engine_used[next] = compiled;
            routed += compiled;
            if (compiled && held) {
                held_ids[nheld++] = next;
            } else if (compiled) {
                pthread_mutex_lock(&cc.mu);
                cc.queue[cc.qtail++] = next;
                pthread_cond_signal(&cc.cv);
                pthread_mutex_unlock(&cc.mu);
            } else {
                ready[nready++] = next;
            }
            next++;
        }
        if (held && next == njobs && nready == 0) {  /* a batch with no interpreter jobs */
            held = 0;
            release_held(&cc, held_ids, nheld);
        }
        /* compiled jobs: launch into free slots, collect finished ones */
        if (nsl) {
            pthread_mutex_lock(&cc.mu);
            if (cc.failed) {
                ok = tc_fail(err, errlen, "%s", cc.err);
                pthread_mutex_unlock(&cc.mu);
                break;
            }
            if (!loads_open && !held && next == njobs && rhead == nready && !pending)
                loads_open = 1;  /* a batch's interpreter has every job it will get */
            /* a batch loads every build that is ready before it launches any of them: the first
               load waits for the device's running work and the others find it idle, where a
               load before each launch would wait for the compiled jobs just launched */
            while (ok && cc.defer && loads_open && cc.rhead < cc.rtail) {
                int id = cc.ready[cc.rhead++];
                pthread_mutex_unlock(&cc.mu);  /* the compile threads go on while this loads */
                double tl = tc_now();
                ok = tc_enum_job_load(jobs[id], &cc.prep[id], err, errlen);
                load_s += tc_now() - tl;
                pthread_mutex_lock(&cc.mu);
                if (ok)
                    loaded[nloaded++] = id;
                progress = 1;
            }
            for (int s = 0; ok && loads_open && s < nsl; s++) {
                if (slot[s].id >= 0)
                    continue;
                int id;
                if (cc.defer) {
                    if (lhead == nloaded)
                        break;
                    id = loaded[lhead++];
                    pthread_mutex_unlock(&cc.mu);
                } else {
                    if (cc.rhead == cc.rtail)
                        break;
                    id = cc.ready[cc.rhead++];
                    pthread_mutex_unlock(&cc.mu);
                    /* loaded by its compile thread: the launch shape */
                    ok = tc_enum_job_load(jobs[id], &cc.prep[id], err, errlen);
                }
                if (ok)
                    ok = tc_enum_job_launch(&cc.prep[id], slot[s].dev, slot[s].host, slot[s].st,
                                            err, errlen) &&
                         tc_cu_check(cudaEventRecord(slot[s].done, slot[s].st), "event", err,
                                     errlen);
                pthread_mutex_lock(&cc.mu);
                if (!ok)
                    break;
                slot[s].id = id;
                start[id] = tc_now() - t0;
                progress = 1;
            }
            pthread_mutex_unlock(&cc.mu);
            for (int s = 0; ok && s < nsl; s++) {
                if (slot[s].id < 0)
                    continue;
                cudaError_t q = cudaEventQuery(slot[s].done);
                if (q == cudaErrorNotReady)
                    continue;
                if (!tc_cu_check(q, "compiled job", err, errlen)) {
                    ok = 0;
                    break;
                }
                int id = slot[s].id;
                tc_enum_job_result(&cc.prep[id], slot[s].host, &results[id]);
                finish[id] = tc_now() - t0;
                slot[s].id = -1;
                finished++;
                progress = 1;
            }
            if (!ok)
                break;
        }
        /* a free stream and admissible jobs: a new wave */
        int s = -1;
        for (int i = 0; i < nst; i++)
            if (!busy[i]) {
                s = i;
                break;
            }
        /* a batch whose interpreter has run out of work takes back the jobs still waiting for a
           compile thread: the GPU is free now, the compile threads are not */
        if (route && !held && s >= 0 && !pending && rhead == nready && next == njobs) {
            pthread_mutex_lock(&cc.mu);
            while (cc.qhead < cc.qtail) {
                int id = cc.queue[--cc.qtail];
                ready[nready++] = id;
                if (engine_used)
                    engine_used[id] = 0;
                taken_back++;
            }
            pthread_mutex_unlock(&cc.mu);
        }
        if (s >= 0 && !pending && rhead < nready && inflight < o.max_inflight_jobs) {
            int n = 0;
            /* a batch's first wave is smaller: the GPU (and the held compiles) start sooner */
            int cap = wave_launched_at < 0 && first_wave > 0 ? first_wave : o.max_wave_jobs;
            while (rhead + n < nready && n < cap && inflight + n < o.max_inflight_jobs)
                n++;
            for (int i = 0; i < n; i++)
                wj[i] = jobs[ready[rhead + i]];
            if (!tc_wave_prepare(&pending, wj, n, err, errlen)) {
                ok = 0;
                break;
            }
            pending_n = n;
            pending_need = tc_wave_bytes(pending);
        }
        /* the prepared wave goes out when a stream is free and its footprint fits */
        if (s >= 0 && pending && (inflight == 0 || bytes + pending_need <= o.max_device_bytes)) {
            int n = pending_n;
            double at = tc_now() - t0;
            if (!tc_wave_launch(pending, st[s], o.share, err, errlen)) {
                tc_wave_free(pending);
                pending = NULL;
                ok = 0;
                break;
            }
            fl[s].w = pending;
            fl[s].ids = tc_xmalloc((size_t)n * sizeof(int));
            memcpy(fl[s].ids, ready + rhead, (size_t)n * sizeof(int));
            fl[s].n = fl[s].left = n;
            fl[s].bytes = pending_need;
            for (int i = 0; i < n; i++)
                start[ready[rhead + i]] = at;
            if (held) {
                held = 0;
                release_held(&cc, held_ids, nheld);
                wave_launched_at = at;
            }
            busy[s] = 1;
            rhead += n;
            inflight += n;
            bytes += pending_need;
            pending = NULL;
            progress = 1;
        }
        /* finished jobs, finished waves */
        for (int i = 0; i < nst; i++) {
            if (!busy[i])
                continue;
            Flight *f = &fl[i];
            for (int k = 0; k < f->n; k++) {
                int id = f->ids[k];
                if (id >= 0 && tc_wave_job_done(f->w, k)) {
                    finish[id] = tc_now() - t0;
                    tc_wave_result(f->w, k, &results[id]);
                    f->ids[k] = -1;
                    f->left--;
                    finished++;
                    inflight--;
                    progress = 1;
                }
            }
            int fin = tc_wave_finished(f->w);
            if (fin < 0) {
                ok = tc_cu_check(cudaEventQuery(0), "serving wave", err, errlen);
                if (ok)
                    ok = tc_fail(err, errlen, "a serving wave failed");
                break;
            }
            if (fin && f->left == 0) {
                bytes -= f->bytes;
                tc_wave_free(f->w);
                free(f->ids);
                memset(f, 0, sizeof *f);
                busy[i] = 0;
                progress = 1;
            }
        }
        if (!progress)
            nap();
    }
    double loop_end = tc_now() - t0;
    pthread_mutex_lock(&cc.mu);
    cc.stop = 1;
    cc.qhead = cc.qtail;  /* nothing more to compile */
    pthread_cond_broadcast(&cc.cv);
    pthread_mutex_unlock(&cc.mu);
    for (int i = 0; i < nthreads; i++)
        pthread_join(tid[i], NULL);
    for (int i = cc.rhead; i < cc.rtail; i++)  /* builds never loaded (after an error) */
        tc_enum_job_drop(&cc.prep[cc.ready[i]]);
    tc_wave_free(pending);
    for (int i = 0; i < nst; i++) {
        if (busy[i]) {
            tc_wave_free(fl[i].w);
            free(fl[i].ids);
        }
        cudaStreamSynchronize(st[i]);
        cudaStreamDestroy(st[i]);
    }
    tc_wave_pool_trim();  /* every wave is done: the device is idle */
    for (int i = 0; i < MAX_COMPILED; i++) {
        if (slot[i].st) {
            cudaStreamSynchronize(slot[i].st);
            cudaStreamDestroy(slot[i].st);
        }
        if (slot[i].done)
            cudaEventDestroy(slot[i].done);
        if (slot[i].dev)
            cudaFree(slot[i].dev);
        if (slot[i].host)
            cudaFreeHost(slot[i].host);
    }
    pthread_mutex_destroy(&cc.mu);
    pthread_cond_destroy(&cc.cv);
    free(cc.prep);
    free(cc.queue);
    free(cc.ready);
    free(ready);
    free(wj);
    free(held_ids);
    free(loaded);
    tc_serve_last_wave_at = wave_launched_at;
    tc_serve_last_routed = routed;
    tc_serve_last_taken_back = taken_back;
    tc_serve_last_compile_busy = cc.busy;
    tc_serve_last_compile_load = load_s;
    tc_serve_last_loop_end = loop_end;
    return ok;
}
