/*
 * The frame server (include/craw/server.h): streams admitted against a
 * device-memory budget, a queue of frames, and one worker thread that
 * keeps the device busy with every frame that has a free slot (earliest
 * deadline first), retires finished frames by polling their events, and runs
 * the AWB loop of the streams that keep a track. A stream's waiting
 * frames are bounded by max_queued: beyond it a submit returns EAGAIN.
 *
 * Locking: one mutex guards everything the worker and the callers share.
 * The worker drops it only around the AWB estimate (host work of a few
 * milliseconds on a stream that has nothing else in flight) and around
 * its short sleeps. Stream creation and destruction are serialised by a
 * second mutex so that the pool's usage before and after a creation is
 * that stream's footprint alone.
 */
#define _POSIX_C_SOURCE 200809L
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include <cuda_runtime_api.h>

#include <craw/server.h>

#include "internal.h"

#define MAX_STREAMS 256
#define MAX_SLOTS 8

struct job {
    struct job *next;
    uint32_t stream;
    const void *src;
    size_t src_pitch;
    void *dst;
    size_t dst_pitch;
    CRAWFrameParams fp;
    double pts;
    uint64_t user;
    uint64_t seq;                    /* submission order within the server */
    int sidx;                        /* its stream's index in streams[] */
    double t_submit, t_launch, due;  /* due: t_submit + the stream's deadline */
    bool noise_measured;             /* the stream's noise model came from this frame */
};

struct slot {
    void *src_dev, *dst_dev;
    size_t src_pitch, dst_pitch;
    cudaEvent_t ev0, ev1;
    struct job *job;                 /* NULL: free */
};

struct stream {
    uint32_t id;
    bool closing;
    CRAWServerStreamParams params;
    CRAWPipeline *pipe;
    cudaStream_t cs;
    uint32_t nb_slots, bpp;
    struct slot slots[MAX_SLOTS];
    uint32_t queued, inflight;
    bool busy_host;                  /* the worker is estimating without the lock */
    uint64_t bytes;
    double last_activity;
    CRAWAwbSmoother *sm;
    bool have_track;
    CRAWIlluminant track;
    bool have_noise;                 /* ESTIMATE_NOISE: measured */
    CRAWNoiseEstimate noise;
};

struct CRAWServer {
    CRAWContext *ctx;                /* private: its pool holds only our streams */
    CRAWServerParams params;
    pthread_mutex_t lock, open_lock;
    pthread_cond_t work_cv, result_cv, idle_cv;
    pthread_t worker;
    bool worker_started, stop;
    struct stream *streams[MAX_STREAMS];
    uint32_t next_id;
    struct job *q_head, *q_tail;
    uint64_t resident;
    CRAWServerResult *results;
    size_t r_head, r_count, r_cap;
    CRAWServerStats stats;
};

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static uint64_t pool_used(CRAWServer *s)
{
    uint64_t v = 0;
    if (cudaMemPoolGetAttribute(s->ctx->pool, cudaMemPoolAttrUsedMemCurrent, &v) != cudaSuccess)
        return 0;
    return v;
}

CRAW_API void craw_server_params_init(CRAWServerParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    p->hbm_budget = 60ull << 30;
    p->max_inflight = 32;
    p->slots_per_stream = 2;
}

CRAW_API void craw_server_stream_params_init(CRAWServerStreamParams *p)
{
    if (!p)
        return;
    memset(p, 0, sizeof(*p));
    craw_pipeline_params_init(&p->pipeline);
    craw_awb_params_init(&p->awb);
    craw_awb_smoother_params_init(&p->smoother);
}

static struct stream *find_stream(CRAWServer *s, uint32_t id)
{
    for (int i = 0; i < MAX_STREAMS; i++)
        if (s->streams[i] && s->streams[i]->id == id)
            return s->streams[i];
    return NULL;
}

/* Frees everything a stream holds; its frames are done. */
static void stream_destroy(CRAWServer *s, struct stream *st)
{
    if (st->cs)
        cudaStreamSynchronize(st->cs);
    for (uint32_t i = 0; i < st->nb_slots; i++) {
        craw_dev_free(s->ctx, st->slots[i].src_dev);
        craw_dev_free(s->ctx, st->slots[i].dst_dev);
        if (st->slots[i].ev0)
            cudaEventDestroy(st->slots[i].ev0);
        if (st->slots[i].ev1)
            cudaEventDestroy(st->slots[i].ev1);
    }
    craw_pipeline_free(&st->pipe);
    craw_awb_smoother_free(&st->sm);
    if (st->cs)
        cudaStreamDestroy(st->cs);
    craw_dev_sync(s->ctx);
    free(st);
}

/* Takes the stream out of the table (lock held) and frees it without the
 * lock; returns with the lock held again. */
static void stream_remove(CRAWServer *s, struct stream *st)
{
    for (int i = 0; i < MAX_STREAMS; i++)
        if (s->streams[i] == st)
            s->streams[i] = NULL;
    s->resident -= st->bytes;
    s->stats.streams--;
    pthread_mutex_unlock(&s->lock);
    pthread_mutex_lock(&s->open_lock);
    stream_destroy(s, st);
    pthread_mutex_unlock(&s->open_lock);
    pthread_mutex_lock(&s->lock);
    pthread_cond_broadcast(&s->idle_cv);
}

static void post_result(CRAWServer *s, const CRAWServerResult *r)
{
    if (s->r_count == s->r_cap) {
        size_t cap = s->r_cap ? 2 * s->r_cap : 256;
        CRAWServerResult *n = malloc(cap * sizeof(*n));
        if (!n)
            return;   /* out of host memory: the result is lost, the stats keep it */
        for (size_t i = 0; i < s->r_count; i++)
            n[i] = s->results[(s->r_head + i) % s->r_cap];
        free(s->results);
        s->results = n;
        s->r_head = 0;
        s->r_cap = cap;
    }
    s->results[(s->r_head + s->r_count) % s->r_cap] = *r;
    s->r_count++;
    pthread_cond_broadcast(&s->result_cv);
}

static void fail_job(CRAWServer *s, struct job *j, int status, double t)
{
    CRAWServerResult r;
    memset(&r, 0, sizeof(r));
    r.user = j->user;
    r.stream = j->stream;
    r.status = status;
    r.queue_ms = (j->t_launch > 0.0 ? j->t_launch : t) - j->t_submit;
    r.latency_ms = t - j->t_submit;
    s->stats.failed++;
    post_result(s, &r);
}

/* Enqueues one frame on its stream (lock held). */
static int launch(CRAWServer *s, struct stream *st, struct slot *sl, struct job *j)
{
    const CRAWPipelineParams *pp = &st->params.pipeline;
    CRAWFrameParams fp = j->fp;
    CRAWImage src = { sl->src_dev, sl->src_pitch, CRAW_FORMAT_R16_UNORM, pp->width, pp->height };
    CRAWImage dst = { sl->dst_dev, sl->dst_pitch, pp->out_format, pp->width, pp->height };
    int ret;

    if ((st->params.flags & CRAW_SERVER_STREAM_AUTO_WB) && st->have_track) {
        fp.wb_mode = CRAW_WB_REBALANCE;
        fp.illuminant = st->track;
    }
    if (cudaEventRecord(sl->ev0, st->cs) != cudaSuccess ||
        cudaMemcpy2DAsync(sl->src_dev, sl->src_pitch, j->src, j->src_pitch, (size_t)pp->width * 2,
                          pp->height, cudaMemcpyDefault, st->cs) != cudaSuccess)
        return CRAW_ERROR(EIO);
    if (st->params.flags & CRAW_SERVER_STREAM_ESTIMATE_NOISE) {
        /* Once per stream; the call waits for the copy above and returns
         * with the estimate (the worker holds the lock meanwhile). */
        if (!st->have_noise) {
            if ((ret = craw_noise_estimate_cuda(&src, fp.profile, NULL, &st->noise, st->cs)) < 0)
                return ret;
            st->have_noise = true;
            j->noise_measured = true;
        }
        if (!(fp.noise_override.a > 0.0f))
            fp.noise_override = st->noise.model;
    }
    if ((ret = craw_pipeline_record(st->pipe, st->cs, &src, &dst, &fp)) < 0)
        return ret;
    if (cudaMemcpy2DAsync(j->dst, j->dst_pitch, sl->dst_dev, sl->dst_pitch,
                          (size_t)pp->width * st->bpp, pp->height, cudaMemcpyDefault,
                          st->cs) != cudaSuccess ||
        cudaEventRecord(sl->ev1, st->cs) != cudaSuccess)
        return CRAW_ERROR(EIO);
    return 0;
}

/* Starts every queued frame that may start (lock held): of the first
 * queued frame of each stream whose stream has a free slot (and, keeping
 * an AWB track, nothing in flight), the one due first, while the device
 * has room; a stream's own frames start in their order. */
static bool launch_ready(CRAWServer *s)
{
    bool progress = false;

    while (s->stats.inflight < s->params.max_inflight) {
        bool seen[MAX_STREAMS] = { false };
        struct job *best = NULL, *best_prev = NULL, *prev = NULL;
        int best_slot = -1;

        for (struct job *j = s->q_head; j; prev = j, j = j->next) {
            struct stream *st = s->streams[j->sidx];
            int si = -1;
            if (seen[j->sidx])
                continue;
            seen[j->sidx] = true;
            if (!st || st->id != j->stream || st->busy_host ||
                ((st->params.flags & CRAW_SERVER_STREAM_AUTO_WB) && st->inflight))
                continue;
            for (uint32_t k = 0; k < st->nb_slots && si < 0; k++)
                if (!st->slots[k].job)
                    si = (int)k;
            if (si >= 0 && (!best || j->due < best->due)) {
                best = j;
                best_prev = prev;
                best_slot = si;
            }
        }
        if (!best)
            break;
        /* Unlink. */
        if (best_prev)
            best_prev->next = best->next;
        else
            s->q_head = best->next;
        if (s->q_tail == best)
            s->q_tail = best_prev;
        s->stats.queued--;
        progress = true;
        best->t_launch = now_ms();
        {
            struct stream *st = s->streams[best->sidx];
            struct slot *sl = &st->slots[best_slot];
            int ret;
            st->queued--;
            if ((ret = launch(s, st, sl, best)) < 0) {
                /* Anything already enqueued for it only touches the slot,
                 * whose next use is ordered after it on the same stream. */
                fail_job(s, best, ret, now_ms());
                free(best);
                st->last_activity = now_ms();
                pthread_cond_broadcast(&s->idle_cv);
                continue;
            }
            sl->job = best;
            st->inflight++;
            s->stats.inflight++;
        }
    }
    return progress;
}

/* The AWB reading of a stream's finished frame, pushed into its track.
 * Called without the lock; the stream is marked busy_host meanwhile. */
static void awb_update(struct stream *st, struct job *j, CRAWServerResult *r)
{
    CRAWAwbHistogram h;
    CRAWIlluminant il;

    if (craw_pipeline_get_awb_histogram(st->pipe, &h) < 0 || !j->fp.profile)
        return;
    if (craw_awb_estimate(j->fp.profile, &h, &st->params.awb, &r->estimate) < 0)
        return;
    if (craw_awb_smoother_push(st->sm, j->pts, &r->estimate, false, &il) == 0) {
        r->awb_valid = true;
        r->awb = il;
        st->track = il;
        st->have_track = true;
    }
}

/* The slot of a stream's oldest frame in flight, or NULL. */
static struct slot *oldest_slot(struct stream *st)
{
    struct slot *o = NULL;
    for (uint32_t k = 0; k < st->nb_slots; k++)
        if (st->slots[k].job && (!o || st->slots[k].job->seq < o->job->seq))
            o = &st->slots[k];
    return o;
}

/* Retires every finished frame (lock held; dropped around AWB work). A
 * stream's frames finish in submission order on its CUDA stream and are
 * retired in that order: the oldest first, and none after one that is
 * still running. */
static bool retire_done(CRAWServer *s)
{
    bool progress = false;

    for (int i = 0; i < MAX_STREAMS; i++) {
        struct stream *st = s->streams[i];
        if (!st)
            continue;
        for (;;) {
            struct slot *sl = oldest_slot(st);
            struct job *j = sl ? sl->job : NULL;
            CRAWServerResult r;
            cudaError_t e;
            float dev_ms = 0.0f;

            if (!j)
                break;
            e = cudaEventQuery(sl->ev1);
            if (e == cudaErrorNotReady)
                break;
            progress = true;
            memset(&r, 0, sizeof(r));
            r.user = j->user;
            r.stream = j->stream;
            r.status = e == cudaSuccess ? 0 : CRAW_ERROR(EIO);
            if (e == cudaSuccess && cudaEventElapsedTime(&dev_ms, sl->ev0, sl->ev1) == cudaSuccess)
                r.device_ms = dev_ms;
            if (j->noise_measured) {
                r.noise_valid = true;
                r.noise = st->noise;
            }
            if (r.status == 0 && (st->params.flags & CRAW_SERVER_STREAM_AUTO_WB)) {
                st->busy_host = true;
                pthread_mutex_unlock(&s->lock);
                awb_update(st, j, &r);
                pthread_mutex_lock(&s->lock);
                st->busy_host = false;
            }
            r.queue_ms = j->t_launch - j->t_submit;
            r.latency_ms = now_ms() - j->t_submit;
            sl->job = NULL;
            st->inflight--;
            s->stats.inflight--;
            if (r.status < 0)
                s->stats.failed++;
            else
                s->stats.completed++;
            st->last_activity = now_ms();
            post_result(s, &r);
            free(j);
            pthread_cond_broadcast(&s->idle_cv);
        }
    }
    return progress;
}

/* Closes streams whose producer has gone quiet (lock held). */
static void reclaim_idle(CRAWServer *s)
{
    const double t = now_ms();
    if (!s->params.idle_timeout_ms)
        return;
    for (int i = 0; i < MAX_STREAMS; i++) {
        struct stream *st = s->streams[i];
        if (st && !st->closing && !st->queued && !st->inflight && !st->busy_host &&
            t - st->last_activity > s->params.idle_timeout_ms) {
            craw_log(s->ctx, CRAW_LOG_WARN, "server: stream %u idle for %u ms, closed\n", st->id,
                     s->params.idle_timeout_ms);
            st->closing = true;
            s->stats.streams_reclaimed++;
            stream_remove(s, st);
        }
    }
}

static void *worker_main(void *arg)
{
    CRAWServer *s = arg;

    cudaSetDevice(s->ctx->device);
    pthread_mutex_lock(&s->lock);
    for (;;) {
        bool progress = retire_done(s);
        progress |= launch_ready(s);
        reclaim_idle(s);
        if (progress)
            continue;
        if (s->stats.inflight) {
            struct timespec ts = { 0, 20000 };
            pthread_mutex_unlock(&s->lock);
            nanosleep(&ts, NULL);
            pthread_mutex_lock(&s->lock);
        } else if (s->stop && !s->stats.queued) {
            break;
        } else {
            struct timespec ts;
            clock_gettime(CLOCK_REALTIME, &ts);
            ts.tv_nsec += 20 * 1000 * 1000;
            if (ts.tv_nsec >= 1000000000) {
                ts.tv_sec++;
                ts.tv_nsec -= 1000000000;
            }
            pthread_cond_timedwait(&s->work_cv, &s->lock, &ts);
        }
    }
    pthread_mutex_unlock(&s->lock);
    return NULL;
}

CRAW_API int craw_server_create(CRAWContext *ctx, const CRAWServerParams *params, CRAWServer **out)
{
    CRAWServer *s;
    CRAWCudaInitParams ip;
    int ret;

    if (!ctx || !params || !out)
        return CRAW_ERROR(EINVAL);
    *out = NULL;
    if (!params->hbm_budget || params->slots_per_stream > MAX_SLOTS)
        return CRAW_ERROR(EINVAL);
    if (!(s = calloc(1, sizeof(*s))))
        return CRAW_ERROR(ENOMEM);
    s->params = *params;
    if (!s->params.max_inflight)
        s->params.max_inflight = 32;
    if (!s->params.slots_per_stream)
        s->params.slots_per_stream = 2;
    memset(&ip, 0, sizeof(ip));
    ip.device = ctx->device;
    if ((ret = craw_context_create(&s->ctx, &ip, &ctx->opts)) < 0) {
        free(s);
        return ret;
    }
    pthread_mutex_init(&s->lock, NULL);
    pthread_mutex_init(&s->open_lock, NULL);
    pthread_cond_init(&s->work_cv, NULL);
    pthread_cond_init(&s->result_cv, NULL);
    pthread_cond_init(&s->idle_cv, NULL);
    s->stats.hbm_budget = params->hbm_budget;
    s->next_id = 1;
    if (pthread_create(&s->worker, NULL, worker_main, s) != 0) {
        craw_server_free(&s);
        return CRAW_ERROR(ENOMEM);
    }
    s->worker_started = true;
    *out = s;
    return 0;
}

CRAW_API void craw_server_free(CRAWServer **ps)
{
    CRAWServer *s;

    if (!ps || !*ps)
        return;
    s = *ps;
    if (s->worker_started) {
        pthread_mutex_lock(&s->lock);
        s->stop = true;
        pthread_cond_broadcast(&s->work_cv);
        pthread_mutex_unlock(&s->lock);
        pthread_join(s->worker, NULL);
    }
    for (int i = 0; i < MAX_STREAMS; i++)
        if (s->streams[i]) {
            stream_destroy(s, s->streams[i]);
            s->streams[i] = NULL;
        }
    while (s->q_head) {
        struct job *j = s->q_head;
        s->q_head = j->next;
        free(j);
    }
    free(s->results);
    pthread_cond_destroy(&s->work_cv);
    pthread_cond_destroy(&s->result_cv);
    pthread_cond_destroy(&s->idle_cv);
    pthread_mutex_destroy(&s->lock);
    pthread_mutex_destroy(&s->open_lock);
    craw_context_free(&s->ctx);
    free(s);
    *ps = NULL;
}

CRAW_API int craw_server_stream_open(CRAWServer *s, const CRAWServerStreamParams *params,
                                     uint32_t *stream_id)
{
    const CRAWPipelineParams *pp;
    struct stream *st;
    uint64_t before, after;
    int ret = 0, free_idx = -1;

    if (!s || !params || !stream_id)
        return CRAW_ERROR(EINVAL);
    pp = &params->pipeline;
    if (!craw_is_out_format(pp->out_format))
        return CRAW_ERROR(EINVAL);
    if ((params->flags & ~(CRAW_SERVER_STREAM_AUTO_WB | CRAW_SERVER_STREAM_ESTIMATE_NOISE)) ||
        ((params->flags & CRAW_SERVER_STREAM_AUTO_WB) && !(pp->flags & CRAW_PIPELINE_FLAG_AWB_HISTOGRAM))) {
        craw_log(s->ctx, CRAW_LOG_ERROR, "server: AUTO_WB needs CRAW_PIPELINE_FLAG_AWB_HISTOGRAM\n");
        return CRAW_ERROR(EINVAL);
    }
    if ((params->flags & CRAW_SERVER_STREAM_ESTIMATE_NOISE) &&
        !(pp->flags & (CRAW_PIPELINE_FLAG_DENOISE | CRAW_PIPELINE_FLAG_TEMPORAL_DENOISE))) {
        craw_log(s->ctx, CRAW_LOG_ERROR, "server: ESTIMATE_NOISE needs a denoising pipeline\n");
        return CRAW_ERROR(EINVAL);
    }
    if (!(st = calloc(1, sizeof(*st))))
        return CRAW_ERROR(ENOMEM);
    st->params = *params;
    st->bpp = (uint32_t)craw_format_bpp(pp->out_format);
    st->nb_slots = s->params.slots_per_stream;

    pthread_mutex_lock(&s->open_lock);
    cudaSetDevice(s->ctx->device);
    craw_dev_sync(s->ctx);
    before = pool_used(s);
    if ((ret = craw_pipeline_create(s->ctx, pp, &st->pipe)) < 0)
        goto fail;
    /* One stream priority for all: priorities by deadline (tried) starve
     * the large frames' kernels behind the small ones' and lengthen the
     * tail of the mix; the deadlines order the launches instead. */
    if (cudaStreamCreateWithFlags(&st->cs, cudaStreamNonBlocking) != cudaSuccess) {
        ret = CRAW_ERROR(ENOMEM);
        goto fail;
    }
    for (uint32_t k = 0; k < st->nb_slots; k++) {
        struct slot *sl = &st->slots[k];
        sl->src_pitch = ((size_t)pp->width * 2 + 255) / 256 * 256;
        sl->dst_pitch = ((size_t)pp->width * st->bpp + 255) / 256 * 256;
        if ((ret = craw_dev_alloc(s->ctx, &sl->src_dev, sl->src_pitch * pp->height)) < 0 ||
            (ret = craw_dev_alloc(s->ctx, &sl->dst_dev, sl->dst_pitch * pp->height)) < 0)
            goto fail;
        if (cudaEventCreate(&sl->ev0) != cudaSuccess || cudaEventCreate(&sl->ev1) != cudaSuccess) {
            ret = CRAW_ERROR(ENOMEM);
            goto fail;
        }
    }
    if ((params->flags & CRAW_SERVER_STREAM_AUTO_WB) &&
        (ret = craw_awb_smoother_create(&params->smoother, &st->sm)) < 0)
        goto fail;
    if ((ret = craw_dev_sync(s->ctx)) < 0)
        goto fail;
    after = pool_used(s);
    st->bytes = after > before ? after - before : 0;

    pthread_mutex_lock(&s->lock);
    for (int i = 0; i < MAX_STREAMS && free_idx < 0; i++)
        if (!s->streams[i])
            free_idx = i;
    if (free_idx < 0 || s->resident + st->bytes > s->params.hbm_budget) {
        ret = free_idx < 0 ? CRAW_ERROR(EMFILE) :
              st->bytes > s->params.hbm_budget ? CRAW_ERROR(ENOSPC) : CRAW_ERROR(EAGAIN);
        s->stats.streams_refused++;
        pthread_mutex_unlock(&s->lock);
        craw_log(s->ctx, CRAW_LOG_VERBOSE, "server: stream of %llu bytes refused (%llu of %llu in use)\n",
                 (unsigned long long)st->bytes, (unsigned long long)s->resident,
                 (unsigned long long)s->params.hbm_budget);
        goto fail;
    }
    st->id = s->next_id++;
    st->last_activity = now_ms();
    s->streams[free_idx] = st;
    s->resident += st->bytes;
    s->stats.streams++;
    s->stats.streams_admitted++;
    *stream_id = st->id;
    pthread_mutex_unlock(&s->lock);
    pthread_mutex_unlock(&s->open_lock);
    return 0;

fail:
    stream_destroy(s, st);
    pthread_mutex_unlock(&s->open_lock);
    return ret;
}

CRAW_API int craw_server_stream_close(CRAWServer *s, uint32_t id)
{
    struct stream *st;

    if (!s)
        return CRAW_ERROR(EINVAL);
    pthread_mutex_lock(&s->lock);
    st = find_stream(s, id);
    if (!st || st->closing) {
        pthread_mutex_unlock(&s->lock);
        return CRAW_ERROR(ENOENT);
    }
    st->closing = true;
    while (st->queued || st->inflight || st->busy_host)
        pthread_cond_wait(&s->idle_cv, &s->lock);
    stream_remove(s, st);
    pthread_mutex_unlock(&s->lock);
    return 0;
}

CRAW_API int craw_server_submit(CRAWServer *s, uint32_t id, const void *src, size_t src_pitch,
                                void *dst, size_t dst_pitch, const CRAWFrameParams *fp, double pts,
                                uint64_t user)
{
    struct stream *st;
    struct job *j;

    if (!s || !src || !dst || !fp)
        return CRAW_ERROR(EINVAL);
    if (!(j = calloc(1, sizeof(*j))))
        return CRAW_ERROR(ENOMEM);
    j->stream = id;
    j->src = src;
    j->src_pitch = src_pitch;
    j->dst = dst;
    j->dst_pitch = dst_pitch;
    j->fp = *fp;
    j->pts = pts;
    j->user = user;
    pthread_mutex_lock(&s->lock);
    st = find_stream(s, id);
    if (!st || st->closing) {
        pthread_mutex_unlock(&s->lock);
        free(j);
        return CRAW_ERROR(ENOENT);
    }
    if (src_pitch < (size_t)st->params.pipeline.width * 2 ||
        dst_pitch < (size_t)st->params.pipeline.width * st->bpp) {
        pthread_mutex_unlock(&s->lock);
        free(j);
        return CRAW_ERROR(EINVAL);
    }
    if (s->params.max_queued && st->queued >= s->params.max_queued) {
        s->stats.submits_refused++;
        pthread_mutex_unlock(&s->lock);
        free(j);
        return CRAW_ERROR(EAGAIN);
    }
    for (int i = 0; i < MAX_STREAMS; i++)
        if (s->streams[i] == st)
            j->sidx = i;
    j->t_submit = now_ms();
    j->due = j->t_submit + (st->params.deadline_ms > 0.0f ? (double)st->params.deadline_ms : 1e12);
    j->seq = s->stats.submitted;
    if (s->q_tail)
        s->q_tail->next = j;
    else
        s->q_head = j;
    s->q_tail = j;
    st->queued++;
    st->last_activity = j->t_submit;
    s->stats.queued++;
    s->stats.submitted++;
    pthread_cond_signal(&s->work_cv);
    pthread_mutex_unlock(&s->lock);
    return 0;
}

CRAW_API int craw_server_poll(CRAWServer *s, CRAWServerResult *out, uint32_t max, int timeout_ms)
{
    uint32_t n = 0;

    if (!s || (!out && max))
        return CRAW_ERROR(EINVAL);
    pthread_mutex_lock(&s->lock);
    if (!s->r_count && timeout_ms != 0) {
        struct timespec ts;
        clock_gettime(CLOCK_REALTIME, &ts);
        if (timeout_ms > 0) {
            ts.tv_sec += timeout_ms / 1000;
            ts.tv_nsec += (long)(timeout_ms % 1000) * 1000000L;
            if (ts.tv_nsec >= 1000000000L) {
                ts.tv_sec++;
                ts.tv_nsec -= 1000000000L;
            }
        }
        while (!s->r_count) {
            if (timeout_ms > 0) {
                if (pthread_cond_timedwait(&s->result_cv, &s->lock, &ts) != 0)
                    break;
            } else {
                pthread_cond_wait(&s->result_cv, &s->lock);
            }
        }
    }
    while (n < max && s->r_count) {
        out[n++] = s->results[s->r_head];
        s->r_head = (s->r_head + 1) % s->r_cap;
        s->r_count--;
    }
    pthread_mutex_unlock(&s->lock);
    return (int)n;
}

CRAW_API int craw_server_drain(CRAWServer *s)
{
    if (!s)
        return CRAW_ERROR(EINVAL);
    pthread_mutex_lock(&s->lock);
    while (s->stats.queued || s->stats.inflight)
        pthread_cond_wait(&s->idle_cv, &s->lock);
    pthread_mutex_unlock(&s->lock);
    return 0;
}

CRAW_API int craw_server_get_stats(CRAWServer *s, CRAWServerStats *out)
{
    if (!s || !out)
        return CRAW_ERROR(EINVAL);
    pthread_mutex_lock(&s->lock);
    *out = s->stats;
    out->hbm_budget = s->params.hbm_budget;
    out->hbm_resident = s->resident;
    pthread_mutex_unlock(&s->lock);
    return 0;
}
