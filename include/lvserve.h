/* lvserve.h -- serving loop: many background-subtraction streams on one GPU.
 *
 * No counterpart in the reference: its applications drive one IBackgroundSubtractor per sequence,
 * one frame at a time (apps/changedet/src/main.cpp:236-344). Here one scheduler thread owns a batch
 * context (lvbgs_batch) and the handles of all streams:
 *
 *   - A stream can be opened at any time. It is admitted -- initialize() runs on the device --
 *     when the device bytes of the resident streams plus its own (lvbgs_device_bytes, plus its share
 *     of the batch work area) fit the HBM budget. Admission is in arrival order.
 *   - Frames can be submitted at any time. Each tick takes the oldest queued frame of every
 *     resident stream that has no frame in flight and launches them as one batched frame step.
 *     Two ticks are kept in flight, so frames that arrive while one runs join the next one
 *     (continuous batching), and the host work of a tick overlaps the device work of the previous.
 *   - A resident stream with no queued frame for idle_spill_ms is spilled to pinned host memory
 *     when its bytes are needed to admit or restore another stream; it is restored when a frame
 *     of it is queued and the budget allows.
 *   - A frame's latency runs from its submission to its mask being in host memory.
 *
 * Every stream's results are identical to driving it alone with lvbgs_apply: frames of one
 * stream run in submission order, and each stream's generator draws depend only on its own seed,
 * frame index and pixel (not on the batch it runs in, nor on spills).
 * All functions are thread-safe; the image and mask buffers of a submitted frame must stay valid
 * until its result has been returned by lvserve_poll (pinned host memory avoids staging copies).
 */
#ifndef LVSERVE_H
#define LVSERVE_H

#include <stddef.h>
#include <stdint.h>

#include "lvbgs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct lvserve_ctx* lvserve_handle;

typedef struct {
    int device_id;
    size_t hbm_budget_bytes;        /* device bytes for resident streams and the batch work area; 0: 80% of free memory */
    size_t host_spill_budget_bytes; /* pinned host bytes for spilled streams; 0: no limit */
    int max_live;                   /* open streams (waiting, resident or spilled); 256 */
    int max_queue;                  /* queued frames per stream before lvserve_submit answers LVBGS_BUSY; 8 */
    double idle_spill_ms;           /* a stream idle this long may be spilled to make room; 500 */
    int max_inflight;               /* ticks in flight, 1..LVBGS_BATCH_MAX_INFLIGHT; 2 */
    int pawcs_lanes;                /* host threads running PAWCS frame steps (and creating / destroying
                                       PAWCS handles) beside the batched ticks, on streams of the lowest
                                       priority (the ticks: the highest); 1 */
} lvserve_config;

typedef struct {
    int stream_id;
    uint64_t tag;      /* the caller's tag of the frame */
    int status;        /* lvbgs_status of the frame step */
    double latency_ms; /* submission -> mask in host memory */
} lvserve_result;

typedef struct {
    uint64_t frames_done, px_done, ticks, admitted, rejected, busy_refusals, spills, restores, closed;
    int live, waiting, resident, spilled;
    size_t device_bytes_in_use; /* resident streams + batch work area, as accounted against the budget */
    size_t peak_device_bytes;
    double mean_tick_streams;   /* streams per tick */
    double busy_ms;             /* wall time with at least one tick (or PAWCS frame step) in flight */
    uint64_t pawcs_frames;      /* frames of PAWCS streams done (on the PAWCS lanes) */
} lvserve_stats;

lvbgs_status lvserve_default_config(lvserve_config* out);
lvbgs_status lvserve_create(const lvserve_config* cfg, lvserve_handle* out);
/* finishes the frames in flight and queued, then frees every stream */
lvbgs_status lvserve_destroy(lvserve_handle s);

/* Opens a stream (BackgroundSubtractorSuBSENSE_ / BackgroundSubtractorPAWCS_ constructor +
 * initialize(img, roi)); the image and roi are copied, and initialize() runs when the stream is
 * admitted. SuBSENSE streams are batched into ticks; PAWCS streams (one or three channels) run frame
 * by frame on the PAWCS lanes. Idle streams of either algorithm spill to pinned host memory when room
 * is needed. LVBGS_BUSY at max_live; LVBGS_BAD_SIZE if the
 * stream alone can never fit the budget. */
lvbgs_status lvserve_open(lvserve_handle s, lvbgs_algo algo, const lvbgs_params* params, const uint8_t* init_image,
                          int width, int height, int channels, size_t stride, const uint8_t* roi, int* stream_id);
/* Queues one frame (apply(img, fgmask, learning_rate)); LVBGS_BUSY if max_queue frames are queued. */
lvbgs_status lvserve_submit(lvserve_handle s, int stream_id, const uint8_t* image, size_t stride, uint8_t* fgmask,
                            double learning_rate, uint64_t tag);
/* Closes a stream once its queued frames are done. */
lvbgs_status lvserve_close(lvserve_handle s, int stream_id);
/* Returns up to max finished frames, waiting up to timeout_ms for the first one. */
int lvserve_poll(lvserve_handle s, lvserve_result* out, int max, int timeout_ms);
/* Waits until no frame is queued or in flight and no stream waits for admission (LVBGS_BUSY on timeout). */
lvbgs_status lvserve_drain(lvserve_handle s, int timeout_ms);
lvbgs_status lvserve_get_stats(lvserve_handle s, lvserve_stats* out);
/* latency quantile (q in [0,1]) of the frames finished since creation or the last reset; -1 if none */
double lvserve_latency_quantile(lvserve_handle s, double q);
lvbgs_status lvserve_reset_stats(lvserve_handle s);
/* 0: resident, 1: waiting for admission, 2: spilled, 3: closed or unknown */
int lvserve_stream_state(lvserve_handle s, int stream_id);
const char* lvserve_last_error(lvserve_handle s);

/* Room planning (the scheduler's policy, exported for tests). Given the bytes in use, the budget,
 * the bytes needed, and n resident candidate streams (their bytes and idle times, in ms), chooses
 * the longest-idle candidates idle at least idle_spill_ms to spill until the need fits. Writes
 * their indices to spill_out and returns how many (0 if the need fits as is), or -1 if it cannot
 * fit even after spilling every eligible candidate (then nothing is chosen). */
int lvserve_plan_room(size_t used, size_t budget, size_t need, const size_t* cand_bytes, const double* cand_idle_ms,
                      int n, double idle_spill_ms, int* spill_out);

/* The serving workload: Poisson stream arrivals, each stream living U[life_min_s, life_max_s]
 * and sending frames at fps; resolutions {320x240, 640x480, 1280x720, 1920x1080} with res_prob;
 * single-channel with gray_prob. Content is the synthetic preset 4 of lvbgs_synth.h, rendered
 * in pinned host memory (pool_frames distinct frames per stream, replayed forth and back). */
typedef struct {
    double duration_s;    /* measured span after warm-up */
    double warmup_s;      /* span before measuring */
    double arrival_rate;  /* new streams per second: 4 */
    double life_min_s, life_max_s; /* 10, 60 */
    double fps;           /* 30 */
    double res_prob[4];   /* .3 .3 .3 .1 */
    double gray_prob;     /* .25 */
    double pawcs_prob;    /* share of the streams (one or three channels) that run PAWCS: .025 */
    int prefill;          /* 1: start from the stationary population (Poisson(rate * mean life) streams with residual lives) */
    int pool_frames;      /* 4 */
    int render_threads;   /* 4 */
    uint64_t seed;
} lvserve_sim_config;

typedef struct {
    double window_s;           /* measured span */
    uint64_t frames;           /* frames finished in the window */
    double mpix_per_s;         /* W*H of those frames per second */
    double frames_per_s;
    double offered_mpix_per_s; /* W*H of the frames submitted in the window per second */
    double p50_ms, p90_ms, p99_ms, max_ms; /* latency of frames submitted in the window */
    double admit_wait_p50_ms, admit_wait_p99_ms; /* open -> admitted */
    double pawcs_p50_ms, pawcs_p99_ms;           /* latency of the PAWCS streams' frames */
    uint64_t pawcs_frames;                       /* PAWCS frames finished in the window */
    double subsense_p50_ms, subsense_p99_ms;     /* latency of the SuBSENSE streams' frames (batched ticks) */
    double mean_live, mean_resident, mean_tick_streams, gpu_busy_frac;
    uint64_t ticks, arrivals, admitted, rejected, dropped, spills, restores, late_frames;
    int peak_live;
    size_t peak_device_bytes;
    int status;                /* first error (lvbgs_status), 0 if none */
} lvserve_sim_result;

lvbgs_status lvserve_default_sim_config(lvserve_sim_config* out);
lvbgs_status lvserve_simulate(const lvserve_config* cfg, const lvserve_sim_config* sim, lvserve_sim_result* out);

#ifdef __cplusplus
}
#endif
#endif
