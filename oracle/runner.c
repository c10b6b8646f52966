/* ORACLE (test infrastructure only): CPU baseline driver.
 *
 * Runs independent SuBSENSE instances, one per stream, on a pool of worker
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
    int next;
    pthread_mutex_t mu;
} job_t;

static void* worker(void* arg) {
    job_t* j = (job_t*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        const int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->n) break;
        osub_params p;
        osub_default_params(&p);
        p.seed = j->seeds[i];
        osub_t* o = osub_create(&p);
        const size_t fb = (size_t)j->w[i] * j->h[i] * j->c[i];
        uint8_t* mask = (uint8_t*)malloc((size_t)j->w[i] * j->h[i]);
        osub_initialize(o, j->frames[i], j->w[i], j->h[i], j->c[i], NULL);
        for (int f = 1; f < j->nf[i]; ++f) osub_apply(o, j->frames[i] + (size_t)f * fb, mask, 0.0);
        if (j->last_masks && j->last_masks[i])
            for (size_t k = 0; k < (size_t)j->w[i] * j->h[i]; ++k) j->last_masks[i][k] = mask[k];
        free(mask);
        osub_destroy(o);
    }
    return NULL;
}

double orun_streams(int n_streams, const uint8_t* const* frames, const int* n_frames, const int* widths,
                    const int* heights, const int* channels, const uint64_t* seeds, int n_threads,
                    uint8_t* const* last_masks) {
    job_t j = {n_streams, frames, n_frames, widths, heights, channels, seeds, last_masks, 0,
               PTHREAD_MUTEX_INITIALIZER};
    if (n_threads < 1) n_threads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)n_threads);
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    for (int t = 0; t < n_threads; ++t) pthread_create(&th[t], NULL, worker, &j);
    for (int t = 0; t < n_threads; ++t) pthread_join(th[t], NULL);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    free(th);
    return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
