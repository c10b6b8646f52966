/* ORACLE (test infrastructure only): CPU baseline drivers.
 *
 * Run independent SuBSENSE / PAWCS / LOBSTER instances, one per stream, on a pool of worker
 * threads, the same per-sequence parallelism as lv::WorkerPool in
 * apps/changedet/src/main.cpp:148-154 (one instance per core across streams).
 */
#define _POSIX_C_SOURCE 200809L
#include "oracle.h"

#include <pthread.h>
#include <stdlib.h>
#include <time.h>

typedef struct {
    int n;
    const uint8_t* const* frames;
    const int *nf, *w, *h, *c;
    const uint64_t* seeds;
    uint8_t* const* last_masks;
    int warm;  /* applied frames per stream before the timed ones (SuBSENSE runner) */
    int next;
    pthread_mutex_t mu;
} job_t;

/* Thread k initializes streams k, k+T, ... and applies their first `warm` frames, then, after a
 * barrier, applies the rest; the returned time covers those frames only (the per-frame throughput of
 * the model after its first frames, without the initialization). */
typedef struct {
    job_t* j;
    int tid, nth;
    pthread_barrier_t* bar;
} pjob_t;

static void* sworker(void* arg) {
    pjob_t* pj = (pjob_t*)arg;
    job_t* j = pj->j;
    int mine = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth) ++mine;
    osub_t** os = (osub_t**)calloc((size_t)(mine > 0 ? mine : 1), sizeof(osub_t*));
    int m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        osub_params p;
        osub_default_params(&p);
        p.seed = j->seeds[i];
        os[m] = osub_create(&p);
        osub_initialize(os[m], j->frames[i], j->w[i], j->h[i], j->c[i], NULL);
        const size_t fb = (size_t)j->w[i] * j->h[i] * j->c[i];
        uint8_t* mask = (uint8_t*)malloc((size_t)j->w[i] * j->h[i]);
        for (int f = 1; f <= j->warm && f < j->nf[i]; ++f) osub_apply(os[m], j->frames[i] + (size_t)f * fb, mask, 0.0);
        free(mask);
    }
    pthread_barrier_wait(pj->bar);
    m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        const size_t fb = (size_t)j->w[i] * j->h[i] * j->c[i];
        uint8_t* mask = (uint8_t*)malloc((size_t)j->w[i] * j->h[i]);
        for (int f = 1 + j->warm; f < j->nf[i]; ++f) osub_apply(os[m], j->frames[i] + (size_t)f * fb, mask, 0.0);
        if (j->last_masks && j->last_masks[i])
            for (size_t k = 0; k < (size_t)j->w[i] * j->h[i]; ++k) j->last_masks[i][k] = mask[k];
        free(mask);
    }
    pthread_barrier_wait(pj->bar);
    for (int k = 0; k < mine; ++k) osub_destroy(os[k]);
    free(os);
    return NULL;
}

double orun_streams(int n_streams, const uint8_t* const* frames, const int* n_frames, const int* widths,
                    const int* heights, const int* channels, const uint64_t* seeds, int n_threads,
                    uint8_t* const* last_masks, int warm_frames) {
    job_t j = {n_streams, frames, n_frames, widths, heights, channels, seeds, last_masks, warm_frames < 0 ? 0 : warm_frames, 0,
               PTHREAD_MUTEX_INITIALIZER};
    if (n_threads < 1) n_threads = 1;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)n_threads + 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    pjob_t* pj = (pjob_t*)malloc(sizeof(pjob_t) * (size_t)n_threads);
    for (int t = 0; t < n_threads; ++t) {
        pj[t] = (pjob_t){&j, t, n_threads, &bar};
        pthread_create(&th[t], NULL, sworker, &pj[t]);
    }
    struct timespec t0, t1;
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t0);
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&bar);
    free(th);
    free(pj);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* PAWCS: the same scheme (PAWCS's model initialization is much heavier than a frame and is not part
 * of the per-frame throughput). */

static void* pworker(void* arg) {
    pjob_t* pj = (pjob_t*)arg;
    job_t* j = pj->j;
    int mine = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth) ++mine;
    opawcs_t** os = (opawcs_t**)calloc((size_t)(mine > 0 ? mine : 1), sizeof(opawcs_t*));
    int m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        opawcs_params p;
        opawcs_default_params(&p);
        p.seed = j->seeds[i];
        os[m] = opawcs_create(&p);
        opawcs_initialize(os[m], j->frames[i], j->w[i], j->h[i], j->c[i], NULL);
    }
    pthread_barrier_wait(pj->bar);
    m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        const size_t fb = (size_t)j->w[i] * j->h[i] * j->c[i];
        uint8_t* mask = (uint8_t*)malloc((size_t)j->w[i] * j->h[i]);
        for (int f = 1; f < j->nf[i]; ++f) opawcs_apply(os[m], j->frames[i] + (size_t)f * fb, mask, 0.0);
        free(mask);
    }
    pthread_barrier_wait(pj->bar);
    for (int k = 0; k < mine; ++k) opawcs_destroy(os[k]);
    free(os);
    return NULL;
}

double orun_pawcs_streams(int n_streams, const uint8_t* const* frames, const int* n_frames, const int* widths,
                          const int* heights, const int* channels, const uint64_t* seeds, int n_threads) {
    job_t j = {n_streams, frames, n_frames, widths, heights, channels, seeds, NULL, 0, 0, PTHREAD_MUTEX_INITIALIZER};
    if (n_threads < 1) n_threads = 1;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)n_threads + 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    pjob_t* pj = (pjob_t*)malloc(sizeof(pjob_t) * (size_t)n_threads);
    for (int t = 0; t < n_threads; ++t) {
        pj[t] = (pjob_t){&j, t, n_threads, &bar};
        pthread_create(&th[t], NULL, pworker, &pj[t]);
    }
    struct timespec t0, t1;
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t0);
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&bar);
    free(th);
    free(pj);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* LOBSTER: the same scheme, at the reference's default learning rate (16) */

static void* lworker(void* arg) {
    pjob_t* pj = (pjob_t*)arg;
    job_t* j = pj->j;
    int mine = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth) ++mine;
    olob_t** os = (olob_t**)calloc((size_t)(mine > 0 ? mine : 1), sizeof(olob_t*));
    int m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        olob_params p;
        olob_default_params(&p);
        p.seed = j->seeds[i];
        os[m] = olob_create(&p);
        olob_initialize(os[m], j->frames[i], j->w[i], j->h[i], j->c[i], NULL);
    }
    pthread_barrier_wait(pj->bar);
    m = 0;
    for (int i = pj->tid; i < j->n; i += pj->nth, ++m) {
        const size_t fb = (size_t)j->w[i] * j->h[i] * j->c[i];
        uint8_t* mask = (uint8_t*)malloc((size_t)j->w[i] * j->h[i]);
        for (int f = 1; f < j->nf[i]; ++f) olob_apply(os[m], j->frames[i] + (size_t)f * fb, mask, 16.0);
        free(mask);
    }
    pthread_barrier_wait(pj->bar);
    for (int k = 0; k < mine; ++k) olob_destroy(os[k]);
    free(os);
    return NULL;
}

double orun_lobster_streams(int n_streams, const uint8_t* const* frames, const int* n_frames, const int* widths,
                            const int* heights, const int* channels, const uint64_t* seeds, int n_threads) {
    job_t j = {n_streams, frames, n_frames, widths, heights, channels, seeds, NULL, 0, 0, PTHREAD_MUTEX_INITIALIZER};
    if (n_threads < 1) n_threads = 1;
    pthread_barrier_t bar;
    pthread_barrier_init(&bar, NULL, (unsigned)n_threads + 1);
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    pjob_t* pj = (pjob_t*)malloc(sizeof(pjob_t) * (size_t)n_threads);
    for (int t = 0; t < n_threads; ++t) {
        pj[t] = (pjob_t){&j, t, n_threads, &bar};
        pthread_create(&th[t], NULL, lworker, &pj[t]);
    }
    struct timespec t0, t1;
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t0);
    pthread_barrier_wait(&bar);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    pthread_barrier_destroy(&bar);
    free(th);
    free(pj);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
