/* lvbgs.h -- C-ABI of the GB300 (sm_103a) SuBSENSE background subtractor.
 *
 * This is the boundary a C++ IBackgroundSubtractor_<lv::CUDA> specialisation (or any FFI)
 * binds to. It replaces the missing CUDA implementation slot of the reference,
 * modules/video/include/litiv/video/BackgroundSubtractionUtils.hpp:136-138
 * ("IBackgroundSubtractor_<lv::CUDA> will not compile here, missing impl") and
 * BackgroundSubtractorLBSP.hpp:77-80 (static_assert(eImpl!=lv::CUDA,"Missing impl")).
 *
 * Conventions: plain pointers and sizes; every call returns an lvbgs_status; the last
 * error message of a handle is available through lvbgs_last_error(). The caller owns all
 * image and mask buffers; a handle owns its model state, which stays resident in device
 * memory between frames. A handle is single-writer (like a reference instance, which is
 * not thread-safe); different handles may be driven from different host threads.
 * Images are 8-bit, 1 or 3 interleaved channels (BGR order is irrelevant to the method),
 * rows `stride` bytes apart. Masks are 8-bit, width*height bytes, 0 or 255.
 * Image and mask pointers may be host (pageable or pinned) or device memory; the library
 * detects which with cudaPointerGetAttributes.
 */
#ifndef LVBGS_H
#define LVBGS_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    LVBGS_OK = 0,
    LVBGS_BAD_ARG = 1,         /* null pointer, bad parameter value (lvAssert_ in the reference) */
    LVBGS_BAD_SIZE = 2,        /* size mismatch with the initialization frame */
    LVBGS_BAD_TYPE = 3,        /* unsupported channel count / type */
    LVBGS_NOT_INITIALIZED = 4, /* apply() before initialize() */
    LVBGS_OOM = 5,             /* device allocation failed */
    LVBGS_DEVICE_TIMEOUT = 6,  /* a bounded device-side wait gave up (kernel returned an error status) */
    LVBGS_DEVICE_ERROR = 7,    /* CUDA runtime error, or no usable sm_103 device */
    LVBGS_UNSUPPORTED = 8,     /* configuration outside what this implementation covers */
    LVBGS_BUSY = 9             /* serving: a queue or capacity limit refused the request (retry later) */
} lvbgs_status;

typedef enum {
    LVBGS_ALGO_SUBSENSE = 0,
    LVBGS_ALGO_PAWCS = 1,
    LVBGS_ALGO_LOBSTER = 2,
    LVBGS_ALGO_VIBE = 3,
    LVBGS_ALGO_PBAS = 4
} lvbgs_algo;

typedef struct lvbgs_ctx* lvbgs_handle;

/* Constructor parameters of BackgroundSubtractorSuBSENSE_ (BackgroundSubtractorSuBSENSE.hpp:52-57,
 * defaults :22-31) and of IBackgroundSubtractorLBSP_ (BackgroundSubtractorLBSP.hpp:46-55, defaults
 * :23-28), plus the seed of the counter-based generator that replaces rand(). */
typedef struct {
    size_t desc_dist_threshold_offset;   /* 3 */
    size_t min_color_dist_threshold;     /* 30 */
    size_t bg_samples;                   /* 50 (this implementation supports 1..64) */
    size_t required_bg_samples;          /* 2 */
    size_t samples_for_moving_avgs;      /* 100 */
    float rel_lbsp_threshold;            /* 0.333f */
    size_t lbsp_threshold_offset;        /* 0 */
    int default_median_blur_kernel_size; /* 9 */
    uint64_t seed;                       /* generator key; streams with different seeds draw independently */
    int device_id;                       /* CUDA device (IParallelAlgo_<CUDA>(bInitUseCUDA, nDeviceID), algo.hpp:82-129) */
    float update_rate;                   /* PBAS: fInitUpdateRate (16), in (0, 255]; unused by the others */
} lvbgs_params;

/* one stream's frame in a batched call */
typedef struct {
    const uint8_t* image; /* width*height*channels bytes, rows `stride` bytes apart (0 = dense) */
    size_t stride;
    uint8_t* fgmask;      /* output, width*height bytes, may be NULL */
    double learning_rate; /* apply()'s learningRateOverride: <=0 uses the internal T(x) (default 0) */
} lvbgs_frame;

/* fills the reference defaults (BackgroundSubtractorSuBSENSE.hpp:22-31) */
lvbgs_status lvbgs_default_params(lvbgs_algo algo, lvbgs_params* out);

/* BackgroundSubtractorSuBSENSE_ constructor (BackgroundSubtractorSuBSENSE.cpp:62-78): checks the
 * parameters (required samples <= samples, one positive threshold, non-negative LBSP threshold)
 * and selects the CUDA device (lv::cuda::init, utils/src/cuda.cpp:18-75). */
lvbgs_status lvbgs_create(lvbgs_algo algo, const lvbgs_params* params, lvbgs_handle* out);
lvbgs_status lvbgs_destroy(lvbgs_handle h);

/* IIBackgroundSubtractor::initialize(img, roi) (BackgroundSubtractionUtils.hpp:29-31,
 * BackgroundSubtractorSuBSENSE.cpp:107-186). roi is NULL (whole frame) or width*height bytes of
 * 0/255 values. Allocates the device model and builds it from the frame (refreshModel(1.0)). */
lvbgs_status lvbgs_initialize(lvbgs_handle h, const uint8_t* image, int width, int height, int channels,
                              size_t stride, const uint8_t* roi);

/* IIBackgroundSubtractor::apply(img, fgmask, learningRateOverride) (BackgroundSubtractorSuBSENSE.cpp:188-612).
 * Enqueues the frame step on `cuda_stream` (a cudaStream_t, NULL = the per-handle stream) and
 * waits for it; fgmask receives the post-processed foreground mask. image and fgmask may be device
 * or host memory. A SuBSENSE or PAWCS mask in page-locked host memory (cudaHostAlloc /
 * cudaHostRegister, mapped at the same address) is written by the post-processing kernel itself
 * over the host link; a mask in pageable host memory is copied from a device staging buffer. */
lvbgs_status lvbgs_apply(lvbgs_handle h, const uint8_t* image, size_t stride, uint8_t* fgmask,
                         double learning_rate, void* cuda_stream);

/* Batched frame step: one frame of each of the n streams (handles on the same device, all
 * initialized). The SuBSENSE streams run in one sequence of phase kernels over a per-stream
 * descriptor table (15 launches per group; large batches run as up to four concurrent groups, see
 * lvbgs_set_batch_groups), enqueued on cuda_stream. The PAWCS streams' frame steps run on their
 * handles' own CUDA streams, forked from cuda_stream and joined back into it, all in flight together;
 * a PAWCS step waits on the host for its fixed-point rounds, so the call returns once every PAWCS
 * step is enqueued to its end (their device errors are returned by this call). Other algorithms are
 * rejected (LVBGS_UNSUPPORTED). Results are identical to n separate lvbgs_apply calls.
 * lvbgs_batch_wait() waits and reports the SuBSENSE part's device errors. Host buffers referenced
 * by `frames` must stay valid until the wait returns. No reference counterpart (the reference runs
 * one subtractor per sequence). */
/* How lvbgs_batch_apply runs large batches (>= 8 streams and >= 4 Mi pixels): G in 2..4 (default 4)
 * splits them into up to G groups of about equal pixels (at least 4 streams each), run on the
 * caller's stream and on further streams of the first handle (forked and joined with events), so
 * that one group's latency-bound phases overlap the others' work; 1 runs every batch as one group
 * (one set of kernels, as the per-kernel timing of lvbgs_debug_set_timing expects). Process-wide. */
lvbgs_status lvbgs_set_batch_groups(int groups);
lvbgs_status lvbgs_batch_apply(const lvbgs_handle* handles, const lvbgs_frame* frames, int n, void* cuda_stream);
lvbgs_status lvbgs_batch_wait(const lvbgs_handle* handles, int n, void* cuda_stream);

/* Batch contexts (serving; no reference counterpart). A context owns the work area of batched
 * frame steps (descriptor tables, repair lists, status), so that a scheduler can batch any subset
 * of streams per tick and keep up to LVBGS_BATCH_MAX_INFLIGHT ticks in flight on one CUDA stream.
 * The frames and masks of a tick in flight should be in pinned host memory (or device memory),
 * so that enqueueing the next tick does not wait for it; a stream may be in at most one tick in
 * flight. Results are identical to lvbgs_apply. */
#define LVBGS_BATCH_MAX_INFLIGHT 4
typedef struct lvbgs_batch_ctx* lvbgs_batch;
/* reserve_px / reserve_streams size the work area (it grows on demand while no tick is in flight) */
lvbgs_status lvbgs_batch_create(int device_id, size_t reserve_px, int reserve_streams, lvbgs_batch* out);
lvbgs_status lvbgs_batch_destroy(lvbgs_batch b);
lvbgs_status lvbgs_batch_reserve(lvbgs_batch b, size_t px, int n_streams);
/* enqueues one tick over n streams on cuda_stream (required, non-NULL); *ticket names it */
/* The repair kernel of this context's ticks is a cooperative launch, which starts only once all of its
 * blocks can be resident; with other work on the device (PAWCS frame steps on other streams, say) a
 * grid of every co-resident block can wait a long time. This gives it 1/divisor of them (default 1). */
lvbgs_status lvbgs_batch_set_repair_share(lvbgs_batch b, int divisor);
lvbgs_status lvbgs_batch_submit(lvbgs_batch b, const lvbgs_handle* handles, const lvbgs_frame* frames, int n,
                                void* cuda_stream, uint64_t* ticket);
/* 1: the tick has completed, 0: not yet, -1: unknown ticket or device error */
int lvbgs_batch_query(lvbgs_batch b, uint64_t ticket);
/* waits for the tick (oldest first) and returns its status, device-side error flags included */
lvbgs_status lvbgs_batch_complete(lvbgs_batch b, uint64_t ticket);

/* getBackgroundImage (BackgroundSubtractorSuBSENSE.cpp:614-630): width*height*channels bytes */
lvbgs_status lvbgs_get_background(lvbgs_handle h, uint8_t* out);
/* getBackgroundDescriptorsImage (BackgroundSubtractorSuBSENSE.cpp:632-649): width*height*channels uint16 */
lvbgs_status lvbgs_get_background_descriptors(lvbgs_handle h, uint16_t* out);
/* refreshModel(fSamplesRefreshFrac, bForceFGUpdate) (BackgroundSubtractorSuBSENSE.cpp:80-105) */
lvbgs_status lvbgs_refresh_model(lvbgs_handle h, float fraction, int force_fg_update);
/* setAutomaticModelReset (BackgroundSubtractionUtils.cpp:24-26) */
lvbgs_status lvbgs_set_automatic_model_reset(lvbgs_handle h, int enabled);
/* getDefaultLearningRate (BackgroundSubtractorSuBSENSE.hpp:69): always 0 */
double lvbgs_get_default_learning_rate(lvbgs_handle h);
/* setROI (BackgroundSubtractionUtils.cpp:38-48) with validateROI (:28-36): the ROI (width*height bytes,
 * host or device memory) loses its 2-pixel border ring and must keep a pixel; on an initialized
 * handle the model is re-initialized from the latest background image with it, otherwise it is kept
 * for the next lvbgs_initialize() of the same size that passes no ROI (which also reuses the last
 * validated ROI, :86-87). */
lvbgs_status lvbgs_set_roi(lvbgs_handle h, const uint8_t* roi, int width, int height);
/* getROICopy (BackgroundSubtractionUtils.cpp:50-52): the validated ROI, width*height bytes */
lvbgs_status lvbgs_get_roi(lvbgs_handle h, uint8_t* out);

/* sizes of an initialized handle */
lvbgs_status lvbgs_get_size(lvbgs_handle h, int* width, int* height, int* channels);
/* device bytes of the model state of a width x height x channels stream of `algo` (admission control;
 * the size of a spill buffer) */
size_t lvbgs_state_bytes(lvbgs_algo algo, int width, int height, int channels, size_t bg_samples);
/* all device bytes an initialized, resident handle holds (model, scratch and its own workspace) */
size_t lvbgs_device_bytes(lvbgs_algo algo, int width, int height, int channels, size_t bg_samples);

/* Moves a stream's whole device state (SuBSENSE or PAWCS) to `host_buffer` (lvbgs_state_bytes()
 * bytes, pinned memory recommended) and frees the device model; lvbgs_restore() uploads it again.
 * The model evolves bit-identically across a spill/restore pair. */
lvbgs_status lvbgs_spill(lvbgs_handle h, void* host_buffer, size_t bytes);
lvbgs_status lvbgs_restore(lvbgs_handle h, const void* host_buffer, size_t bytes);

/* LBSP::compute2 dense descriptor extraction on the device (modules/features2d/src/LBSP.cpp:102-152,
 * LBSP.hpp:70-77). abs_threshold >= 0 selects LBSP(size_t) (absolute threshold), otherwise
 * LBSP(rel_threshold, offset). desc: width*height*channels uint16; the 2-pixel border is left as is. */
lvbgs_status lvbgs_lbsp_compute2(const uint8_t* image, int width, int height, int channels, long abs_threshold,
                                 float rel_threshold, size_t offset, uint16_t* desc, int device_id);

/* Same computation as lvbgs_lbsp_compute2, for callers that must not allocate device memory
 * (a real-time thread with a no-allocation rule, a process held to a fixed GPU memory budget).
 * No counterpart in the reference. It allocates nothing: the image and descriptors are staged in
 * one file-scope device array of 24 MiB, so width*height*channels may not exceed 8,388,608
 * (LVBGS_BAD_SIZE otherwise). The CUDA runtime reserves that array, and loads the LBSP kernel,
 * when the library's modules are first used on a device (lazy module loading is the default), so
 * the FIRST call on a device is the one that may allocate: make it during set-up, before any
 * stream capture, or run with CUDA_MODULE_LOADING=EAGER. The array then stays on every GPU that
 * used it until the process exits (or the application resets the device). All calls share the one
 * array: calls that overlap on the GPU (from several host threads, or on streams that run
 * concurrently) race and must be serialised by the caller. cuda_stream must belong to device_id
 * (NULL: the default stream); the call returns after its work there completed, and the caller's
 * current device is left as it was. */
lvbgs_status lvbgs_lbsp_compute2_noalloc(const uint8_t* image, int width, int height, int channels,
                                         long abs_threshold, float rel_threshold, size_t offset, uint16_t* desc,
                                         int device_id, void* cuda_stream);

/* Change-detection evaluation on the device (modules/datasets: lv::BinClassif::accumulate,
 * src/metrics.cpp:21-61). Adds to counts[6] = {TP, TN, FP, FN, shadow errors, don't care} the
 * classification of a foreground mask (255 = positive) against CDnet-coded ground truth (255
 * positive, 0 negative, 85 out of scope and 170 unknown = don't care, 50 shadow) and an optional ROI
 * (0 = don't care). width*height bytes each, host or device memory; gt NULL counts every pixel as
 * don't care. Runs on cuda_stream (NULL: the default stream) and returns after it. */
lvbgs_status lvbgs_classif_accumulate(const uint8_t* fgmask, const uint8_t* gt, const uint8_t* roi, int width,
                                      int height, uint64_t counts[6], int device_id, void* cuda_stream);
/* lv::BinClassifMetrics (include/litiv/datasets/metrics.hpp:203-256) of counts[6]: out[8] = recall,
 * specificity, false positive rate, false negative rate, percentage of bad classifications,
 * precision, F-measure, Matthews correlation coefficient (0 where a denominator is 0). */
lvbgs_status lvbgs_classif_metrics(const uint64_t counts[6], double out[8]);

/* last error message of a handle (or of the library when h is NULL) */
const char* lvbgs_last_error(lvbgs_handle h);

/* ---- inspection (parity tests and tools): model state in the reference's layout ----
 * `which` takes the map ids below; the layout is the reference's: one full-frame map per
 * quantity, interleaved channels, and N sample images for the sample maps. */
enum {
    LVBGS_MAP_R = 0, LVBGS_MAP_V, LVBGS_MAP_T, LVBGS_MAP_DLAST, LVBGS_MAP_DMIN_LT, LVBGS_MAP_DMIN_ST,
    LVBGS_MAP_RAW_LT, LVBGS_MAP_RAW_ST, LVBGS_MAP_FIN_LT, LVBGS_MAP_FIN_ST, /* float [H*W] */
    LVBGS_MAP_UNSTABLE, LVBGS_MAP_BLINKS, LVBGS_MAP_LAST_RAW_FG, LVBGS_MAP_LAST_FG,
    LVBGS_MAP_LAST_FG_DIL_INV, LVBGS_MAP_LAST_RAW_BLINK, LVBGS_MAP_ROI,     /* uint8 [H*W] */
    LVBGS_MAP_LAST_COLOR,                                                    /* uint8 [H*W*C] */
    LVBGS_MAP_LAST_DESC,                                                     /* uint16 [H*W*C] */
    LVBGS_MAP_SAMPLE_COLOR,                                                  /* uint8 [N][H*W*C] */
    LVBGS_MAP_SAMPLE_DESC,                                                   /* uint16 [N][H*W*C] */
    LVBGS_MAP_DS_LT, LVBGS_MAP_DS_ST,                                        /* float [H/8*W/8*C] */
    LVBGS_MAP_LUT,                                                           /* uint8 [256] */
    LVBGS_MAP_SAMPLE_GRAD,                                                   /* PBAS: uint8 [N][H*W*C] */
    LVBGS_MAP_GRAD,                                                          /* PBAS: uint8 [H*W*C] */
    LVBGS_MAP_MEAN_GRAD,                                                     /* PBAS: float [1] */
    LVBGS_MAP_COUNT
};
lvbgs_status lvbgs_debug_map_bytes(lvbgs_handle h, int which, size_t* bytes);
lvbgs_status lvbgs_debug_get_map(lvbgs_handle h, int which, void* out, size_t bytes);

/* frame-level scalars of a stream */
typedef struct {
    uint64_t frame_idx, frames_since_last_reset, model_reset_cooldown;
    int32_t auto_model_reset_enabled, learning_rate_scaling_enabled, use_3x3_spread, median_blur_kernel_size;
    float lr_lower_cap, lr_upper_cap, last_nonzero_desc_ratio;
    uint64_t nonzero_desc_count, tot_color_diff;
    uint64_t n_relevant_px, orig_roi_px;
    uint64_t stat_samples_evaluated, stat_sample_writes; /* cumulative, for the algorithmic-byte count */
    uint64_t stat_repair_rounds, stat_repair_rematched;  /* cumulative raster-order repair work */
} lvbgs_scalars;
lvbgs_status lvbgs_get_scalars(lvbgs_handle h, lvbgs_scalars* out);

/* Per-kernel timing of frame steps (inspection): lvbgs_debug_set_timing(h, batched, n) records CUDA
 * events around each kernel of the next n steps launched by h (batched != 0: the batched steps it
 * leads; 0 disables); lvbgs_debug_tick_profile() waits for them and returns the average duration in
 * ms of each kernel, in launch order: evaluation, long sample scans, ghost resolution, repair, commit/closing, row runs,
 * vertical unions, holes, erosion/combination, median row-window counts, median, frame-level epilogue,
 * dilation/blinks,
 * automatic model reset, frame close. Returns the number of values written. */
lvbgs_status lvbgs_debug_set_timing(lvbgs_handle h, int batched, int n_ticks);
int lvbgs_debug_tick_profile(lvbgs_handle h, int batched, double* out_ms, int max_n);
/* Phase durations (microseconds) of the repair kernel of the last step launched by h (batched != 0:
 * its last batched step): the device timer at kernel entry and after every grid barrier, as
 * differences: re-match of round 0, re-resolution of round 0, re-match of round 1, ...; then the
 * number of re-matched pixels of each round. Waits for the device. Returns the number of values
 * written. */
int lvbgs_debug_repair_phases(lvbgs_handle h, int batched, double* out_us, int max_n);

/* Failure detection (tests): no counterpart in the reference. Makes one of the device-side bounded
 * waits of h's next frame step (lvbgs_apply, or a batched step h leads) run out, so that the path that
 * gives up can be tested without a fault: the kernels return and the call reports the status below;
 * the model state of the streams in that step is then undefined (initialize them again), and the
 * context and every other handle stay usable. One-shot.
 *   LVBGS_FAULT_BARRIER_TIMEOUT  the repair kernel's grid barrier waits 2 ms for a CTA that never
 *                                arrives, then gives up: LVBGS_DEVICE_TIMEOUT
 *   LVBGS_FAULT_REPAIR_LIMIT     the raster-order repair may run no round: LVBGS_DEVICE_ERROR when the
 *                                frame needs one
 *   LVBGS_FAULT_PAWCS_ROUNDS     PAWCS's fixed point may run one round: LVBGS_DEVICE_ERROR when the
 *                                frame needs more */
enum { LVBGS_FAULT_NONE = 0, LVBGS_FAULT_BARRIER_TIMEOUT = 1, LVBGS_FAULT_REPAIR_LIMIT = 2, LVBGS_FAULT_PAWCS_ROUNDS = 3 };
lvbgs_status lvbgs_debug_inject_fault(lvbgs_handle h, int kind);
/* Host time (ms) of the last PAWCS frame step's parts (inspection; no reference counterpart):
 * [0] enqueueing the fixed-point rounds (the first batch and any further ones), [1] the waits for
 * the rounds, [2] enqueueing the rest of the frame step (with the camera-motion decision's wait every
 * 8 or 16 frames), [3] the final wait, [4] the status read-back. */
lvbgs_status lvbgs_debug_pawcs_host_timing(lvbgs_handle h, double* out_ms);

/* ---- PAWCS (BackgroundSubtractorPAWCS, modules/video/src/BackgroundSubtractorPAWCS.cpp) ----
 * A handle created with LVBGS_ALGO_PAWCS runs PAWCS on single-channel (:608-934) and three-channel
 * (:935-1299) frames. lvbgs_params maps onto the constructor (BackgroundSubtractorPAWCS.hpp:47-51):
 * desc_dist_threshold_offset (2), min_color_dist_threshold (20), bg_samples = nMaxNbWords (50; at most
 * 51 for single-channel and 50 for three-channel frames), samples_for_moving_avgs (100),
 * rel_lbsp_threshold (0.333); required_bg_samples is unused.
 * initialize/apply/get_background/get_background_descriptors/get_roi work as for SuBSENSE; batched
 * steps and spilling are SuBSENSE-only for now. */

/* refreshModel(nBaseOccCount, fOccDecrFrac, bForceFGUpdate) (BackgroundSubtractorPAWCS.cpp:107-429) */
lvbgs_status lvbgs_pawcs_refresh_model(lvbgs_handle h, size_t base_occ, float occ_decr_frac, int force_fg_update);

typedef struct {
    uint64_t frame_idx, frames_since_last_reset, model_reset_cooldown, lword_weight_offset;
    int32_t auto_model_reset_enabled, using_moving_camera, median_blur_kernel_size, n_local_words, n_global_words;
    float last_nonflat_ratio;
    uint64_t n_relevant_px, orig_roi_px, ds_roi_px;
    uint64_t fixed_point_rounds; /* local-pass rounds of the last frame step */
} lvbgs_pawcs_scalars;
lvbgs_status lvbgs_pawcs_get_scalars(lvbgs_handle h, lvbgs_pawcs_scalars* out);

/* model state export for parity checks (layouts: float [H*W] maps; uint8 [H*W] masks; LW_* planes
 * [n_relevant_px * local words], ROI pixels in raster order, slot-minor, OCC/FIRST/LAST as uint64; GW:
 * 20 bytes per pool word (colour u8, 3 pad, descriptor u16, 4 pad, bits u8, pad, weight f32, slot i32);
 * GW_MAP float [G][H/2*W/2]; GLUT uint8 [H*W][G]) */
enum {
    LVBGS_PAWCS_MAP_R = 0, LVBGS_PAWCS_MAP_V, LVBGS_PAWCS_MAP_T, LVBGS_PAWCS_MAP_DMIN_LT, LVBGS_PAWCS_MAP_DMIN_ST,
    LVBGS_PAWCS_MAP_RAW_LT, LVBGS_PAWCS_MAP_RAW_ST, LVBGS_PAWCS_MAP_FIN_LT, LVBGS_PAWCS_MAP_FIN_ST,
    LVBGS_PAWCS_MAP_ILLUM, LVBGS_PAWCS_MAP_UNSTABLE, LVBGS_PAWCS_MAP_BLINKS, LVBGS_PAWCS_MAP_LAST_RAW_FG,
    LVBGS_PAWCS_MAP_LAST_FG, LVBGS_PAWCS_MAP_LAST_FG_DIL, LVBGS_PAWCS_MAP_LAST_RAW_BLINK, LVBGS_PAWCS_MAP_ROI,
    LVBGS_PAWCS_MAP_LAST_COLOR, LVBGS_PAWCS_MAP_LAST_DESC, LVBGS_PAWCS_MAP_DS_LT, LVBGS_PAWCS_MAP_DS_ST,
    LVBGS_PAWCS_MAP_LUT, LVBGS_PAWCS_MAP_LW_COLOR, LVBGS_PAWCS_MAP_LW_DESC, LVBGS_PAWCS_MAP_LW_OCC,
    LVBGS_PAWCS_MAP_LW_FIRST, LVBGS_PAWCS_MAP_LW_LAST, LVBGS_PAWCS_MAP_GW, LVBGS_PAWCS_MAP_GW_MAP,
    LVBGS_PAWCS_MAP_GLUT
};
size_t lvbgs_pawcs_debug_export_bytes(lvbgs_handle h, int which);
lvbgs_status lvbgs_pawcs_debug_export(lvbgs_handle h, int which, void* out, size_t bytes);

/* ---- Frame precaching: lv::DataPrecacher (modules/datasets/include/litiv/datasets/utils.hpp:456-478,
 * modules/datasets/src/utils.cpp:302-470) for a GPU consumer ----
 * A loader fills packet `idx` into `dst` (capacity `cap` bytes) and returns its size, 0 at the end of the
 * stream (an empty packet halts precaching, utils.hpp:458), or a size above `cap` for an error. With
 * precaching started, a worker thread loads the packets after the last request into a ring of pinned
 * host slots, each uploaded to its own device slot on a dedicated copy stream, so the uploads of the
 * next packets overlap the caller's work on the current one. */
typedef size_t (*lvbgs_packet_loader)(void* user, size_t idx, uint8_t* dst, size_t cap);
typedef struct lvbgs_precacher_ctx* lvbgs_precacher;
/* DataPrecacher(lDataLoaderCallback) (utils.cpp:302-308); packets are at most max_packet_bytes */
lvbgs_status lvbgs_precacher_create(lvbgs_packet_loader loader, void* user, size_t max_packet_bytes, int device_id,
                                    lvbgs_precacher* out);
/* a precacher over packets already in the caller's host memory: packet idx < count is the packet_bytes
 * bytes at packets + idx * packet_bytes, uploaded from there (no loader, no copy into the ring; pinned
 * memory for asynchronous uploads); the memory must stay valid while the precacher lives */
lvbgs_status lvbgs_precacher_create_host(const uint8_t* packets, size_t packet_bytes, size_t count, int device_id,
                                         lvbgs_precacher* out);
/* ~DataPrecacher(): stops the worker, waits for the device and frees the slots */
lvbgs_status lvbgs_precacher_destroy(lvbgs_precacher p);
/* startAsyncPrecaching(nSuggestedBufferSize) (utils.cpp:358-374): an empty ring of
 * buffer_bytes / max_packet_bytes slots (2 to 64), filled from packet 0 on; a ring of the same size as the
 * last one is reused (allocating pinned slots is slow); 0 leaves precaching off */
lvbgs_status lvbgs_precacher_start(lvbgs_precacher p, size_t buffer_bytes);
/* stopAsyncPrecaching() (utils.cpp:376-386): joins the worker and empties the ring (its slots stay
 * allocated); reports a loader error the worker met (the reference rethrows it) */
lvbgs_status lvbgs_precacher_stop(lvbgs_precacher p);
/* getPacket(idx) (utils.cpp:314-356): *device_packet / *host_packet receive the packet's device and pinned
 * host copies and *size its size (0 and null pointers past the end of the stream). cuda_stream (a
 * cudaStream_t, NULL = the legacy default stream) is made to wait for the packet's upload; no host wait
 * when it is already loaded. The packet stays valid until the next call with another index, which
 * releases it on that call's stream: work enqueued there before the call may still read it. Requests are
 * expected in order; another index restarts the sequence there. When the loader fails, the packets
 * loaded before are still served and the request of the failing one reports the error. Not to be called
 * concurrently. */
lvbgs_status lvbgs_precacher_get(lvbgs_precacher p, size_t idx, void* cuda_stream, const uint8_t** device_packet,
                                 const uint8_t** host_packet, size_t* size);
/* isActive() and getLastReqIdx() (utils.hpp:468-471); SIZE_MAX before the first request */
int lvbgs_precacher_is_active(lvbgs_precacher p);
size_t lvbgs_precacher_last_index(lvbgs_precacher p);
/* a loader over packets already in host memory: user points to an lvbgs_host_packets; packet idx is the
 * packet_bytes bytes at base + idx * packet_bytes, for idx < count */
typedef struct {
    const uint8_t* base;
    size_t packet_bytes;
    size_t count;
} lvbgs_host_packets;
size_t lvbgs_precache_copy_loader(void* user, size_t idx, uint8_t* dst, size_t cap);

/* ---- LOBSTER (BackgroundSubtractorLOBSTER, modules/video/src/BackgroundSubtractorLOBSTER.cpp) ----
 * A handle created with LVBGS_ALGO_LOBSTER runs LOBSTER's non-parallel path (:459-581) on single- and
 * three-channel frames; the reference's GLSL path is not part of this library. lvbgs_params maps onto
 * the constructor (BackgroundSubtractorLOBSTER.hpp:50-55): desc_dist_threshold_offset carries
 * nDescDistThreshold (4), min_color_dist_threshold nColorDistThreshold (30), bg_samples (35, at most 64),
 * required_bg_samples (2), lbsp_threshold_offset (0), rel_lbsp_threshold (0.333); samples_for_moving_avgs
 * is unused. lvbgs_apply's learning_rate is LOBSTER's dLearningRate: it must be positive (ceil() gives
 * the update rate; +inf never updates) and the reference's default is 16 (lvbgs_get_default_learning_rate).
 * initialize, get_background, get_background_descriptors, refresh_model (refreshModel(frac, force),
 * :410-440), set_roi, get_roi, get_size, get_scalars (frame_idx counts apply() calls) and the maps
 * LVBGS_MAP_LAST_FG, _ROI, _LAST_COLOR, _LAST_DESC, _SAMPLE_COLOR, _SAMPLE_DESC and _LUT work as for
 * SuBSENSE; batched steps and spilling are SuBSENSE/PAWCS-only. LOBSTER keeps no frame counter of its own,
 * so draw k of pixel p in the i-th apply() is keyed by frame i (initialize() and refreshes before the first
 * apply() are frame 0). */

/* ---- PBAS (BackgroundSubtractorPBAS, modules/video/src/BackgroundSubtractorPBAS.cpp) ----
 * A handle created with LVBGS_ALGO_PBAS runs BackgroundSubtractorPBAS_1ch on single-channel frames
 * (:61-273) and BackgroundSubtractorPBAS_3ch on three-channel frames (:287-496), with the header's
 * configuration (self diffusion, no R2 acceleration, no advanced morphology; BackgroundSubtractorPBAS.hpp:41-46).
 * lvbgs_params: min_color_dist_threshold carries nInitColorDistThreshold (30), update_rate
 * fInitUpdateRate (16, in (0, 255]), bg_samples (35, at most 64), required_bg_samples (2); the others are
 * unused (the median blur is 9x9 as in the reference). lvbgs_initialize takes no ROI (a non-null roi is
 * LVBGS_UNSUPPORTED); lvbgs_apply's learning_rate is learningRateOverride: when positive it replaces
 * ceil(T(x)), otherwise each pixel uses its own update rate (lvbgs_get_default_learning_rate returns the
 * reference's default, -1). The frame-level mean gradient distance (20 at creation) is kept across
 * initialize() calls, as the reference keeps m_fFormerMeanGradDist. get_background, get_size, get_scalars and
 * the maps LVBGS_MAP_SAMPLE_COLOR, _SAMPLE_GRAD, _R (R(x)), _T (T(x)), _DMIN_LT (D(x)), _GRAD (the last
 * frame's gradient image), _MEAN_GRAD and _ROI work as above; refresh_model, set_roi, background
 * descriptors, batched steps and spilling are LVBGS_UNSUPPORTED. Draws are keyed like ViBe's. */

/* ---- ViBe (BackgroundSubtractorViBe, modules/video/src/BackgroundSubtractorViBe.cpp) ----
 * A handle created with LVBGS_ALGO_VIBE runs BackgroundSubtractorViBe_1ch on single-channel frames
 * (:57-103) and BackgroundSubtractorViBe_3ch on three-channel frames (:112-191), with the header's
 * configuration (L2 colour distance, no single-channel validation, BackgroundSubtractorViBe.hpp:47-52).
 * lvbgs_params: min_color_dist_threshold carries nColorDistThreshold (20), bg_samples (20, at most 64),
 * required_bg_samples (2); the others are unused. lvbgs_initialize takes no ROI (ViBe has none; a
 * non-null roi is LVBGS_UNSUPPORTED); lvbgs_apply's learning_rate must be positive (default 16);
 * get_background, get_size, get_scalars and the maps LVBGS_MAP_SAMPLE_COLOR and _ROI work as above;
 * refresh_model, set_roi, background descriptors, batched steps and spilling are LVBGS_UNSUPPORTED.
 * Draws are keyed like LOBSTER's (frame i = the i-th apply(); initialize() draws sample s of pixel p
 * as draw s of p in frame 0). */

#ifdef __cplusplus
}
#endif
#endif /* LVBGS_H */
