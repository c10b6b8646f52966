/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's SuBSENSE, PAWCS, LOBSTER, ViBe and PBAS per-pixel background
 * subtraction (plstcharles/litiv, modules/video/src/BackgroundSubtractorSuBSENSE.cpp,
 * BackgroundSubtractorPAWCS.cpp, BackgroundSubtractorLOBSTER.cpp, BackgroundSubtractorViBe.cpp,
 * BackgroundSubtractorPBAS.cpp) and of
 * the LBSP descriptor
 * (modules/features2d/include/litiv/features2d/LBSP.hpp).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it,
 * always as the checker.
 *
 * Parity pins: the LBSP descriptor is pinned by the reference's golden vector
 * (modules/features2d/test/data/test_lbsp.bin, see tests/golden/). The SuBSENSE and PAWCS
 * (and LOBSTER, ViBe, PBAS) restatements are pinned to the reference itself: oracle/refshim/build_ref.py compiles the
 * reference's own modules/video/src sources (against a project-written OpenCV stand-in, with rand()
 * routed to the same generator) into oracle/_ref/libref.so, which exposes this same API (rsub_* /
 * rpawcs_*), and tests/test_oracle_reference.py compares every map bit for bit. The OpenCV image
 * operations use one set of definitions on both sides (written from OpenCV's documentation); their
 * parity with a real OpenCV build is unpinned (OpenCV is not installed). Each function cites the
 * reference lines it restates.
 */
#ifndef LV_ORACLE_H
#define LV_ORACLE_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct osub osub_t;

typedef struct {
    size_t desc_dist_threshold_offset;   /* BGSSUBSENSE_DEFAULT_DESC_DIST_THRESHOLD_OFFSET = 3 */
    size_t min_color_dist_threshold;     /* = 30 */
    size_t bg_samples;                   /* = 50 */
    size_t required_bg_samples;          /* = 2 */
    size_t samples_for_moving_avgs;      /* = 100 */
    float rel_lbsp_threshold;            /* = 0.333f */
    size_t lbsp_threshold_offset;        /* = 0 */
    int default_median_blur_kernel_size; /* = 9 */
    uint64_t seed;                       /* key of the counter-based generator */
} osub_params;

/* scalars of the frame-level state, for parity checks */
typedef struct {
    uint64_t frame_idx, frames_since_last_reset, model_reset_cooldown;
    int32_t auto_model_reset_enabled, learning_rate_scaling_enabled, use_3x3_spread, median_blur_kernel_size;
    float lr_lower_cap, lr_upper_cap, last_nonzero_desc_ratio;
    uint64_t nonzero_desc_count, tot_color_diff;
    uint64_t n_relevant_px, orig_roi_px;
    uint64_t stat_samples_evaluated, stat_sample_writes;  /* for the algorithmic-byte count */
} osub_scalars;

enum {
    OSUB_MAP_R = 0, OSUB_MAP_V, OSUB_MAP_T, OSUB_MAP_DLAST, OSUB_MAP_DMIN_LT, OSUB_MAP_DMIN_ST,
    OSUB_MAP_RAW_LT, OSUB_MAP_RAW_ST, OSUB_MAP_FIN_LT, OSUB_MAP_FIN_ST,           /* float [H*W]   */
    OSUB_MAP_UNSTABLE, OSUB_MAP_BLINKS, OSUB_MAP_LAST_RAW_FG, OSUB_MAP_LAST_FG,
    OSUB_MAP_LAST_FG_DIL_INV, OSUB_MAP_LAST_RAW_BLINK, OSUB_MAP_ROI,             /* uint8 [H*W]   */
    OSUB_MAP_LAST_COLOR,                                                           /* uint8 [H*W*C] */
    OSUB_MAP_LAST_DESC,                                                            /* uint16 [H*W*C] */
    OSUB_MAP_SAMPLE_COLOR,                                                         /* uint8 [N][H*W*C] */
    OSUB_MAP_SAMPLE_DESC,                                                          /* uint16 [N][H*W*C] */
    OSUB_MAP_DS_LT, OSUB_MAP_DS_ST,                                                /* float [H/8*W/8*C] */
    OSUB_MAP_LUT,                                                                  /* uint8 [256] */
    OSUB_MAP_COUNT
};

/* error codes (0 = ok) */
#define OSUB_OK 0
#define OSUB_EBADARG 1
#define OSUB_ENOTINIT 2
#define OSUB_EUNSUPPORTED 3

void osub_default_params(osub_params* p);
osub_t* osub_create(const osub_params* p);
void osub_destroy(osub_t* o);
/* BackgroundSubtractorSuBSENSE::initialize (BackgroundSubtractorSuBSENSE.cpp:107-186); roi may be NULL */
int osub_initialize(osub_t* o, const uint8_t* img, int width, int height, int channels, const uint8_t* roi);
/* BackgroundSubtractorSuBSENSE::apply (BackgroundSubtractorSuBSENSE.cpp:188-612) */
int osub_apply(osub_t* o, const uint8_t* img, uint8_t* fgmask, double learning_rate_override);
/* BackgroundSubtractorSuBSENSE::refreshModel (BackgroundSubtractorSuBSENSE.cpp:80-105) */
int osub_refresh_model(osub_t* o, float frac, int force_fg);
int osub_get_background(const osub_t* o, uint8_t* out);               /* :614-630 */
int osub_set_roi(osub_t* o, const uint8_t* roi, int width, int height); /* BackgroundSubtractionUtils.cpp:38-48 */
int osub_get_background_descriptors(const osub_t* o, uint16_t* out);  /* :632-649 */
void osub_set_automatic_model_reset(osub_t* o, int enabled);          /* BackgroundSubtractionUtils.cpp:24-26 */
const void* osub_map(const osub_t* o, int which, size_t* nbytes);
void osub_get_scalars(const osub_t* o, osub_scalars* s);

/* LBSP::compute2 dense extraction (modules/features2d/src/LBSP.cpp:102-152).
 * abs_threshold >= 0 selects the absolute-threshold variant, otherwise the relative
 * one (rel_threshold, abs offset). Border pixels (2 px) are left untouched. */
void olbsp_compute2(const uint8_t* img, int width, int height, int channels,
                    long abs_threshold, float rel_threshold, size_t offset, uint16_t* desc);

/* sampling helpers with border 2 (getSamplePosition_7x7_std2, getNeighborPosition_3x3/_5x5), for
 * the property tests of utils/test/opencv.cpp:390-429 */
void osample_pos_7x7(int rnd, int x0, int y0, int width, int height, int* sx, int* sy);
void oneighbor_pos(int rnd, int use3x3, int x0, int y0, int width, int height, int* nx, int* ny);

/* raw generator access, for the known-answer test */
void ophilox_block(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* ---- PAWCS (modules/video/src/BackgroundSubtractorPAWCS.cpp) ---- */
typedef struct opawcs opawcs_t;

typedef struct {
    size_t desc_dist_threshold_offset;   /* BGSPAWCS_DEFAULT_DESC_DIST_THRESHOLD_OFFSET = 2 */
    size_t min_color_dist_threshold;     /* = 20 */
    size_t max_words;                    /* BGSPAWCS_DEFAULT_MAX_NB_WORDS = 50 (global: max/2) */
    size_t samples_for_moving_avgs;      /* = 100 */
    float rel_lbsp_threshold;            /* = 0.333f */
    size_t lbsp_threshold_offset;        /* = 0 */
    int default_median_blur_kernel_size; /* = 9 */
    uint64_t seed;
} opawcs_params;

typedef struct {
    uint64_t frame_idx, frames_since_last_reset, model_reset_cooldown, lword_weight_offset;
    int32_t auto_model_reset_enabled, using_moving_camera, median_blur_kernel_size, n_local_words, n_global_words;
    float last_nonflat_ratio;
    uint64_t n_relevant_px, orig_roi_px, ds_roi_px;
    uint64_t stat_words_scanned, stat_gdict_events, stat_nb_updates;
} opawcs_scalars;

enum {
    OPAWCS_MAP_R = 0, OPAWCS_MAP_V, OPAWCS_MAP_T, OPAWCS_MAP_DMIN_LT, OPAWCS_MAP_DMIN_ST, OPAWCS_MAP_RAW_LT,
    OPAWCS_MAP_RAW_ST, OPAWCS_MAP_FIN_LT, OPAWCS_MAP_FIN_ST,                         /* float [H*W] */
    OPAWCS_MAP_ILLUM, OPAWCS_MAP_UNSTABLE, OPAWCS_MAP_BLINKS, OPAWCS_MAP_LAST_RAW_FG, OPAWCS_MAP_LAST_FG,
    OPAWCS_MAP_LAST_FG_DIL, OPAWCS_MAP_LAST_RAW_BLINK, OPAWCS_MAP_ROI,                 /* uint8 [H*W] */
    OPAWCS_MAP_LAST_COLOR, OPAWCS_MAP_LAST_DESC,                                     /* [H*W*C] u8 / u16 */
    OPAWCS_MAP_DS_LT, OPAWCS_MAP_DS_ST,                                              /* float [H/8*W/8*C] */
    OPAWCS_MAP_LUT,                                                                  /* uint8 [256] */
    OPAWCS_MAP_LW_COLOR, OPAWCS_MAP_LW_DESC,                                         /* [n_rel*L][C] u8 / u16 */
    OPAWCS_MAP_LW_OCC, OPAWCS_MAP_LW_FIRST, OPAWCS_MAP_LW_LAST,                      /* uint64 [n_rel*L] */
    OPAWCS_MAP_GW,      /* per pool word: colour u8[3], pad, desc u16[3], bits u8, pad, weight f32, slot i32 */
    OPAWCS_MAP_GW_MAP,  /* float [G][H/2*W/2], by pool word */
    OPAWCS_MAP_GLUT,    /* uint8 [H*W][G]: per-pixel global word order (pool indices) */
    OPAWCS_MAP_COUNT
};

void opawcs_default_params(opawcs_params* p);
opawcs_t* opawcs_create(const opawcs_params* p);
void opawcs_destroy(opawcs_t* o);
/* BackgroundSubtractorPAWCS::initialize (BackgroundSubtractorPAWCS.cpp:431-557) */
int opawcs_initialize(opawcs_t* o, const uint8_t* img, int width, int height, int channels, const uint8_t* roi);
/* BackgroundSubtractorPAWCS::apply (:559-1516) */
int opawcs_apply(opawcs_t* o, const uint8_t* img, uint8_t* fgmask, double learning_rate_override);
/* BackgroundSubtractorPAWCS::refreshModel(nBaseOccCount, fOccDecrFrac, bForceFGUpdate) (:107-429) */
int opawcs_refresh_model(opawcs_t* o, size_t base_occ, float occ_decr_frac, int force_fg);
int opawcs_get_background(const opawcs_t* o, uint8_t* out);               /* :1518-1545 */
int opawcs_set_roi(opawcs_t* o, const uint8_t* roi, int width, int height);
int opawcs_get_background_descriptors(const opawcs_t* o, uint16_t* out);  /* :1547-1594 */
void opawcs_set_automatic_model_reset(opawcs_t* o, int enabled);
int opawcs_export(const opawcs_t* o, int which, void* out, size_t bytes);
size_t opawcs_export_bytes(const opawcs_t* o, int which);
void opawcs_get_scalars(const opawcs_t* o, opawcs_scalars* s);

/* ---- LOBSTER (modules/video/src/BackgroundSubtractorLOBSTER.cpp, the non-parallel path) ---- */
typedef struct olob olob_t;

typedef struct {
    size_t desc_dist_threshold;          /* BGSLOBSTER_DEFAULT_DESC_DIST_THRESHOLD = 4 */
    size_t color_dist_threshold;         /* BGSLOBSTER_DEFAULT_COLOR_DIST_THRESHOLD = 30 */
    size_t bg_samples;                   /* BGSLOBSTER_DEFAULT_NB_BG_SAMPLES = 35 */
    size_t required_bg_samples;          /* BGSLOBSTER_DEFAULT_REQUIRED_NB_BG_SAMPLES = 2 */
    float rel_lbsp_threshold;            /* BGSLBSP_DEFAULT_LBSP_REL_SIMILARITY_THRESHOLD = 0.333f */
    size_t lbsp_threshold_offset;        /* = 0 */
    int default_median_blur_kernel_size; /* BGSLBSP_DEFAULT_MEDIAN_BLUR_KERNEL_SIZE = 9 */
    uint64_t seed;
} olob_params;

typedef struct {
    uint64_t frames; /* apply() calls since initialize() (the generator's frame) */
    uint64_t n_relevant_px, orig_roi_px;
    uint64_t stat_samples_evaluated, stat_sample_writes;
} olob_scalars;

enum {
    OLOB_MAP_LAST_FG = 0, OLOB_MAP_ROI,             /* uint8 [H*W] */
    OLOB_MAP_LAST_COLOR, OLOB_MAP_LAST_DESC,        /* [H*W*C] u8 / u16 */
    OLOB_MAP_SAMPLE_COLOR, OLOB_MAP_SAMPLE_DESC,    /* [N][H*W*C] u8 / u16 */
    OLOB_MAP_LUT,                                   /* uint8 [256] */
    OLOB_MAP_COUNT
};

void olob_default_params(olob_params* p);
olob_t* olob_create(const olob_params* p);
void olob_destroy(olob_t* o);
/* BackgroundSubtractorLOBSTER::initialize (BackgroundSubtractorLOBSTER.cpp:442-457) */
int olob_initialize(olob_t* o, const uint8_t* img, int width, int height, int channels, const uint8_t* roi);
/* BackgroundSubtractorLOBSTER::apply (:459-581); learning_rate > 0 (the reference's default is 16) */
int olob_apply(olob_t* o, const uint8_t* img, uint8_t* fgmask, double learning_rate);
/* BackgroundSubtractorLOBSTER::refreshModel (:410-440) */
int olob_refresh_model(olob_t* o, float frac, int force_fg);
int olob_get_background(const olob_t* o, uint8_t* out);              /* :583-600 */
int olob_get_background_descriptors(const olob_t* o, uint16_t* out); /* :602-620 */
const void* olob_map(const olob_t* o, int which, size_t* nbytes);
void olob_get_scalars(const olob_t* o, olob_scalars* s);

/* ---- ViBe (modules/video/src/BackgroundSubtractorViBe.cpp: _1ch for one channel, _3ch for three) ---- */
typedef struct ovibe ovibe_t;
typedef struct {
    size_t color_dist_threshold; /* BGSVIBE_DEFAULT_COLOR_DIST_THRESHOLD = 20 */
    size_t bg_samples;           /* BGSVIBE_DEFAULT_NB_BG_SAMPLES = 20 */
    size_t required_bg_samples;  /* BGSVIBE_DEFAULT_REQUIRED_NB_BG_SAMPLES = 2 */
    uint64_t seed;
} ovibe_params;
void ovibe_default_params(ovibe_params* p);
ovibe_t* ovibe_create(const ovibe_params* p);
void ovibe_destroy(ovibe_t* o);
/* initialize (BackgroundSubtractorViBe.cpp:57-75 / :112-134) */
int ovibe_initialize(ovibe_t* o, const uint8_t* img, int width, int height, int channels);
/* apply (:77-103 / :136-191); learning_rate > 0 (the reference's default is 16) */
int ovibe_apply(ovibe_t* o, const uint8_t* img, uint8_t* fgmask, double learning_rate);
int ovibe_get_background(const ovibe_t* o, uint8_t* out); /* :33-48 */
/* the samples, [N][H*W*C] */
const void* ovibe_samples(const ovibe_t* o, size_t* nbytes);
/* apply() calls, samples evaluated, sample writes */
void ovibe_get_stats(const ovibe_t* o, uint64_t out[3]);

/* ---- PBAS (modules/video/src/BackgroundSubtractorPBAS.cpp: _1ch for one channel, _3ch for three) ---- */
typedef struct opbas opbas_t;
typedef struct {
    size_t color_dist_threshold; /* BGSPBAS_DEFAULT_COLOR_DIST_THRESHOLD = 30 */
    float update_rate;           /* BGSPBAS_DEFAULT_LEARNING_RATE = 16 */
    size_t bg_samples;           /* BGSPBAS_DEFAULT_NB_BG_SAMPLES = 35 */
    size_t required_bg_samples;  /* BGSPBAS_DEFAULT_REQUIRED_NB_BG_SAMPLES = 2 */
    uint64_t seed;
} opbas_params;
enum { OPBAS_MAP_SAMPLE_COLOR = 0, OPBAS_MAP_SAMPLE_GRAD, /* uint8 [N][H*W*C] */
       OPBAS_MAP_R, OPBAS_MAP_T, OPBAS_MAP_D,            /* float [H*W] */
       OPBAS_MAP_GRAD,                                   /* uint8 [H*W*C]: the last frame's gradient image */
       OPBAS_MAP_COUNT };
void opbas_default_params(opbas_params* p);
opbas_t* opbas_create(const opbas_params* p);
void opbas_destroy(opbas_t* o);
/* initialize (BackgroundSubtractorPBAS.cpp:61-109 / :287-324) */
int opbas_initialize(opbas_t* o, const uint8_t* img, int width, int height, int channels);
/* apply (:111-281 / :326-496); learning_rate_override <= 0 uses T(x) (the reference's default is -1) */
int opbas_apply(opbas_t* o, const uint8_t* img, uint8_t* fgmask, double learning_rate_override);
int opbas_get_background(const opbas_t* o, uint8_t* out); /* :36-51 */
const void* opbas_map(const opbas_t* o, int which, size_t* nbytes);
/* m_fFormerMeanGradDist */
float opbas_mean_grad(const opbas_t* o);
/* the gradient image of a frame (GaussianBlur 3x3, Scharr, convertScaleAbs, addWeighted) */
void opbas_gradient(const uint8_t* img, int width, int height, int channels, uint8_t* out);

/* CPU baseline for LOBSTER: as orun_streams (apply phase timed, learning rate 16) */
double orun_lobster_streams(int n_streams, const uint8_t* const* frames, const int* n_frames,
                            const int* widths, const int* heights, const int* channels,
                            const uint64_t* seeds, int n_threads);

/* CPU baseline: runs n independent SuBSENSE instances (one per stream) over their
 * frame sequences on n_threads workers (streams k, k+T, ... on worker k, like the
 * per-sequence lv::WorkerPool of apps/changedet/src/main.cpp:148-154).
 * frames[i] holds n_frames[i] frames of widths[i]*heights[i]*channels[i] bytes;
 * the first frame initializes, the others are applied. Returns the wall time in
 * seconds of the apply phase after the first warm_frames applied frames of every
 * instance (untimed); masks may be NULL. */
double orun_streams(int n_streams, const uint8_t* const* frames, const int* n_frames,
                    const int* widths, const int* heights, const int* channels,
                    const uint64_t* seeds, int n_threads, uint8_t* const* last_masks, int warm_frames);

/* CPU baseline for PAWCS: as orun_streams, timing the apply phase only (after every instance is
 * initialized) */
double orun_pawcs_streams(int n_streams, const uint8_t* const* frames, const int* n_frames,
                          const int* widths, const int* heights, const int* channels,
                          const uint64_t* seeds, int n_threads);

#ifdef __cplusplus
}
#endif
#endif
