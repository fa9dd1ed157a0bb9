/* Serving with continuous batching: jobs arrive over time (an arrival time per job), are admitted
   by footprint as device memory and in-flight slots free up, and run in waves: each wave is the
   batched engine's persistent kernel over the jobs admitted together, on one of several streams,
   with a share of the GPU's blocks so that a newer wave starts while older ones still run.  A job
   is finished the moment its last work unit is (the kernel raises a flag in host-mapped memory),
   not when its wave ends, so a small job that shares a wave with a large one is not held back.

   The host loop never blocks on the device: it admits, launches, polls the flags and frees.
   Compilation is the LUT mapping of the batched engine, done per wave in host threads; a job's
   mapped program is the same whoever shares its wave, so results do not depend on the mix. */
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

#define MAX_STREAMS 8

typedef struct {
    TcWave *w;
    int    *ids;      /* job numbers of the wave */
    int     n, left;  /* jobs, jobs not finished */
    size_t  bytes;
    int     stream;
} Flight;

static void nap(void)
{
    struct timespec t = {0, 20000};  /* 20 us */
    nanosleep(&t, NULL);
}

int cuda_serve_run(const Enum *const *jobs, const double *arrival, int njobs,
                   const CudaServeOpts *opts, double *start, double *finish, EnumResult *results,
                   char *err, size_t errlen)
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
    cudaStream_t st[MAX_STREAMS];
    int busy[MAX_STREAMS];
    for (int s = 0; s < o.streams; s++) {
        busy[s] = 0;
        if (!tc_cu_check(cudaStreamCreateWithFlags(&st[s], cudaStreamNonBlocking), "stream", err,
                         errlen))
            return 0;
    }
    Flight fl[MAX_STREAMS];
    memset(fl, 0, sizeof fl);
    int next = 0, finished = 0, inflight = 0, ok = 1;
    size_t bytes = 0;
    int *ready = tc_xmalloc((size_t)njobs * sizeof *ready), nready = 0, rhead = 0;
    const Enum **wj = tc_xmalloc((size_t)njobs * sizeof *wj);
    TcWave *pending = NULL;  /* a wave prepared but not yet admitted */
    int pending_n = 0;
    size_t pending_need = 0;
    double t0 = tc_now();
    while (ok && finished < njobs) {
        double now = tc_now() - t0;
        while (next < njobs && arrival[next] <= now)
            ready[nready++] = next++;
        /* a free stream and admissible jobs: a new wave */
        int s = -1;
        for (int i = 0; i < o.streams; i++)
            if (!busy[i]) {
                s = i;
                break;
            }
        if (s >= 0 && !pending && rhead < nready && inflight < o.max_inflight_jobs) {
            int n = 0;
            while (rhead + n < nready && n < o.max_wave_jobs && inflight + n < o.max_inflight_jobs)
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
            fl[s].stream = s;
            for (int i = 0; i < n; i++)
                start[ready[rhead + i]] = at;
            busy[s] = 1;
            rhead += n;
            inflight += n;
            bytes += pending_need;
            pending = NULL;
        }
        /* finished jobs, finished waves */
        int progress = 0;
        for (int i = 0; i < o.streams; i++) {
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
    tc_wave_free(pending);
    for (int i = 0; i < o.streams; i++) {
        if (busy[i]) {
            tc_wave_free(fl[i].w);
            free(fl[i].ids);
        }
        cudaStreamSynchronize(st[i]);
        cudaStreamDestroy(st[i]);
    }
    free(ready);
    free(wj);
    return ok;
}
