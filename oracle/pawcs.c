/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * Plain-C restatement of BackgroundSubtractorPAWCS (plstcharles/litiv,
 * modules/video/src/BackgroundSubtractorPAWCS.cpp, header
 * modules/video/include/litiv/video/BackgroundSubtractorPAWCS.hpp) with its base classes
 * (BackgroundSubtractionUtils.cpp, BackgroundSubtractorLBSP.cpp). It keeps the reference's
 * sequential raster scan and floating-point operation order (build with -ffp-contract=off).
 *
 * The reference keeps its words in pools and points at them from per-pixel dictionaries; every
 * local word is referenced by exactly one dictionary slot, so here each slot holds its word by
 * value (a swap of pointers is a swap of words). Global words keep their pool identity (0..G-1),
 * because the per-pixel sort tables point at them: the dictionary and the per-pixel tables hold
 * pool indices.
 *
 * The 1-channel neighbour update works on a copy of the neighbour's word
 * (BackgroundSubtractorPAWCS.cpp:838, `LocalWord_1ch oNeighborLocalWord = ...`), so only its
 * weight sum and its draws have effects; this restatement keeps that behaviour. The 3-channel
 * update works on a reference (:1188) and modifies the neighbour's words.
 *
 * rand() is the counter-based generator of philox.h, keyed by (seed, frame, pixel, draw index);
 * the draw index restarts at 0 each frame and continues from the apply loop into the frame's
 * automatic model reset. OpenCV calls are the definitions of common.h plus those stated below;
 * their parity with the real OpenCV is unpinned.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"
#include "philox.h"

/* constants of BackgroundSubtractorPAWCS.cpp:25-73 */
#define FEEDBACK_R_VAR (0.01f)
#define FEEDBACK_V_INCR (1.000f)
#define FEEDBACK_V_DECR (0.100f)
#define FEEDBACK_T_DECR (0.2500f)
#define FEEDBACK_T_INCR (0.5000f)
#define FEEDBACK_T_LOWER (1.0000f)
#define FEEDBACK_T_UPPER (256.00f)
#define UNSTABLE_REG_RATIO_MIN (0.100f)
#define UNSTABLE_REG_RDIST_MIN (3.000f)
#define LBSPDESC_RATIO_MIN (0.100f)
#define LBSPDESC_RATIO_MAX (0.500f)
#define FRAMELEVEL_DOWNSAMPLE_RATIO 8
#define FRAMELEVEL_MIN_L1DIST_THRES 45
#define FRAMELEVEL_MIN_CDIST_THRES (FRAMELEVEL_MIN_L1DIST_THRES / 10)
#define GWORD_LOOKUP_MAPS_DOWNSAMPLE_RATIO 2
#define GWORD_DEFAULT_NB_INIT_SAMPL_PASSES 2
#define GWORD_DESC_THRES_BITS_MATCH_FACTOR 4
#define DEFAULT_FRAME_AREA (320 * 240)
#define DEFAULT_RESAMPLING_RATE 16
#define DEFAULT_BOOTSTRAP_WIN_SIZE 500
#define DEFAULT_LWORD_WEIGHT_OFFSET (DEFAULT_BOOTSTRAP_WIN_SIZE * 2)
#define DEFAULT_LWORD_OCC_INCR 1
#define DEFAULT_LWORD_MAX_WEIGHT (1.0f)
#define FLAT_REGION_BIT_COUNT 2 /* s_nDescMaxDataRange_1ch/8 */

typedef struct {
    uint8_t color[3];
    uint16_t desc[3];
    uint64_t occ, first, last;
    int valid; /* dictionary slot holds a word (all do after initialization) */
} olword;

struct opawcs {
    opawcs_params p;
    int initialized;
    int W, H, C;
    size_t npx, n_rel, orig_roi;
    uint8_t* roi;
    size_t* pxlut;  /* model index -> pixel */
    size_t* model;  /* pixel -> model index */
    uint8_t lut[256];
    uint64_t frame_idx, frames_since_reset, cooldown, lword_offset;
    int auto_reset, moving_cam, median_k;
    size_t L, G;
    float last_nonflat_ratio;
    int ds_w, ds_h, gw_w, gw_h;
    size_t ds_roi_count;
    uint8_t* ds_roi;
    float *R, *V, *T, *DminLT, *DminST, *RawLT, *RawST, *FinLT, *FinST;
    float *dsLT, *dsST;
    uint8_t* dsframe;
    uint8_t *illum, *unstable, *blinks, *lastRawFG, *lastFG, *lastFGdil, *lastFGdilInv, *lastRawBlink;
    uint8_t *currBlink, *preflood, *holes, *tmp8, *tmp8b, *visited, *raw;
    uint16_t* colcnt;
    int* bfs;
    uint8_t* lastColor;
    uint16_t* lastDesc;
    olword* lw; /* [n_rel * L] */
    /* global words by pool identity */
    uint8_t gw_color[64][3];
    uint16_t gw_desc[64][3];
    uint8_t gw_bits[64];
    float gw_weight[64];
    float* gw_map;     /* [G][gw_w*gw_h] */
    int gdict[64];     /* dictionary slot -> pool index (-1: empty during initialization) */
    int gnext;         /* next unused pool word */
    uint8_t* glut;     /* [npx][G] pool indices, sorted per pixel */
    uint32_t* kctr;
    uint32_t cache_px, cache_blk, cache_out[4];
    int cache_valid;
    uint64_t st_words_scanned, st_gdict_events, st_nb_updates;
};

/* one rand() call of the reference, attributed to pixel px */
static int pdraw(opawcs_t* o, size_t px) {
    const uint32_t p32 = (uint32_t)px;
    const uint32_t k = o->kctr[px]++;
    const uint32_t blk = k >> 2;
    if (!o->cache_valid || o->cache_px != p32 || o->cache_blk != blk) {
        const uint32_t ctr[4] = {blk, p32, (uint32_t)o->frame_idx, 0u};
        const uint32_t key[2] = {(uint32_t)o->p.seed, (uint32_t)(o->p.seed >> 32)};
        ophilox4x32_10(ctr, key, o->cache_out);
        o->cache_px = p32;
        o->cache_blk = blk;
        o->cache_valid = 1;
    }
    return (int)(o->cache_out[k & 3u] & 0x7fffffffu);
}
static void reset_draws(opawcs_t* o) {
    memset(o->kctr, 0, o->npx * sizeof(uint32_t));
    o->cache_valid = 0;
}

/* lv::cdist<3> for unsigned bytes, math.hpp:474-496 */
static size_t cdist3(const uint8_t* curr, const uint8_t* bg) {
    int nonconst = 0, nonnull = curr[0] != bg[0];
    for (int c = 1; c < 3; ++c) {
        nonconst |= (curr[c] != curr[c - 1]) || (bg[c] != bg[c - 1]);
        nonnull |= curr[c] != bg[c];
    }
    if (!nonconst || !nonnull) return 0;
    uint64_t cs = 0, bs = 0, mix = 0;
    for (int c = 0; c < 3; ++c) {
        cs += (uint64_t)(curr[c] * curr[c]);
        bs += (uint64_t)(bg[c] * bg[c]);
        mix += (uint64_t)(curr[c] * bg[c]);
    }
    const float sq = (float)(cs - (mix * mix) / (bs > 1 ? bs : 1));
    return (size_t)sqrtf(sq);
}
/* lv::L1dist<3> of two byte arrays (math.hpp:226-250, the overloads taking pointers and std::arrays):
 * the sum accumulates in its Tout = decltype(L1dist(uchar, uchar)) = unsigned char, so it wraps
 * modulo 256. Every three-channel colour L1 of the path goes through it (directly, :1006, :1179, or
 * through cmixdist, :294, :367, :1085, :1122). */
static size_t l1dist3(const uint8_t* a, const uint8_t* b) {
    return (uint8_t)(absdiff(a[0], b[0]) + absdiff(a[1], b[1]) + absdiff(a[2], b[2]));
}
/* lv::cmixdist, math.hpp:596-605 */
static size_t cmixdist3(const uint8_t* a, const uint8_t* b) { return l1dist3(a, b) / 2 + cdist3(a, b) * 4; }
static size_t hdist3(const uint16_t* a, const uint16_t* b) {
    return popc16(a[0] ^ b[0]) + popc16(a[1] ^ b[1]) + popc16(a[2] ^ b[2]);
}
static unsigned popc3(const uint16_t* d) { return popc16(d[0]) + popc16(d[1]) + popc16(d[2]); }

/* GetLocalWordWeight, BackgroundSubtractorPAWCS.cpp:1596-1598 */
static float lword_weight(const olword* w, uint64_t t, uint64_t off) {
    return (float)w->occ / (float)((w->last - w->first) + (t - w->last) * 2 + off);
}

/* per-pixel thresholds (:633-634 for one channel, :1011-1012 for three) */
static void thresholds(const opawcs_t* o, size_t px, size_t* colorThr, size_t* descThr) {
    const float R = o->R[px];
    const size_t base = ((size_t)1 << (size_t)floorf(R + 0.5f)) + o->p.desc_dist_threshold_offset +
                        (size_t)o->unstable[px] * o->p.desc_dist_threshold_offset;
    /* the reference's unqualified sqrt of a float is the C library's double sqrt (only <cmath> is in
     * scope, whose global namespace has no float overload), and the product is taken in double */
    if (o->C == 1) {
        *colorThr = (size_t)(sqrt((double)R) * (double)o->p.min_color_dist_threshold) / 2;
        *descThr = base;
    } else {
        *colorThr = (size_t)(sqrt((double)R) * (double)o->p.min_color_dist_threshold) * 3;
        *descThr = base * 3;
    }
}

void opawcs_default_params(opawcs_params* p) {
    /* BackgroundSubtractorPAWCS.hpp:22-29, BackgroundSubtractorLBSP.hpp:23-28 */
    p->desc_dist_threshold_offset = 2;
    p->min_color_dist_threshold = 20;
    p->max_words = 50;
    p->samples_for_moving_avgs = 100;
    p->rel_lbsp_threshold = 0.333f;
    p->lbsp_threshold_offset = 0;
    p->default_median_blur_kernel_size = 9;
    p->seed = 0;
}

static void pfree_state(opawcs_t* o) {
    void* ptrs[] = {o->roi,    o->pxlut,  o->model,   o->ds_roi,  o->R,         o->V,         o->T,
                    o->DminLT, o->DminST, o->RawLT,   o->RawST,   o->FinLT,     o->FinST,     o->dsLT,
                    o->dsST,   o->dsframe, o->illum,  o->unstable, o->blinks,   o->lastRawFG, o->lastFG,
                    o->lastFGdil, o->lastFGdilInv, o->lastRawBlink, o->currBlink, o->preflood, o->holes,
                    o->tmp8,   o->tmp8b,  o->visited, o->raw,     o->colcnt,    o->bfs,       o->lastColor,
                    o->lastDesc, o->lw,   o->gw_map,  o->glut,    o->kctr};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    opawcs_params p = o->p;
    memset(o, 0, sizeof(*o));
    o->p = p;
}

opawcs_t* opawcs_create(const opawcs_params* p) {
    /* constructor check, BackgroundSubtractorPAWCS.cpp:105 (m_nMaxGlobalWords = max/2 > 0) */
    if (!p || p->max_words / 2 == 0 || p->max_words > 128) return NULL;
    if (!(p->rel_lbsp_threshold >= 0)) return NULL;
    opawcs_t* o = (opawcs_t*)calloc(1, sizeof(opawcs_t));
    o->p = *p;
    return o;
}

void opawcs_destroy(opawcs_t* o) {
    if (!o) return;
    pfree_state(o);
    free(o);
}

void opawcs_set_automatic_model_reset(opawcs_t* o, int enabled) { o->auto_reset = enabled ? 1 : 0; }

/* floodFill((0,0), 255) + bitwise_not on a 0/255 mask: 255 at 0-pixels not 4-connected to (0,0) */
static void pflood_holes(opawcs_t* o, const uint8_t* pre, uint8_t* holes) {
    const int W = o->W, H = o->H;
    memset(o->visited, 0, o->npx);
    if (pre[0] == 0) {
        int head = 0, tail = 0;
        o->bfs[tail++] = 0;
        o->visited[0] = 1;
        while (head < tail) {
            const int i = o->bfs[head++];
            const int x = i % W, y = i / W;
            const int nb[4][2] = {{x - 1, y}, {x + 1, y}, {x, y - 1}, {x, y + 1}};
            for (int n = 0; n < 4; ++n) {
                const int xx = nb[n][0], yy = nb[n][1];
                if (xx < 0 || yy < 0 || xx >= W || yy >= H) continue;
                const int j = yy * W + xx;
                if (!o->visited[j] && pre[j] == 0) {
                    o->visited[j] = 1;
                    o->bfs[tail++] = j;
                }
            }
        }
    }
    for (size_t i = 0; i < o->npx; ++i) holes[i] = (pre[i] == 0 && !o->visited[i]) ? 255 : 0;
}

/* cv::resize(src, dst, (dw, dh), INTER_AREA) of an 8-bit image (resize_area_u8, oracle/common.h) */
static int resize_area_int(const uint8_t* src, int W, int H, int C, uint8_t* dst, int dw, int dh) {
    return resize_area_u8(src, W, H, C, dst, dw, dh);
}

/* cv::blur(src, dst, 3x3, BORDER_REPLICATE) on CV_32F: normalized box filter whose sums run in
 * double (OpenCV's sum type for float input): per row s = v[x-1] + v[x] + v[x+1], per column
 * t = s[y-1] + s[y] + s[y+1], dst = (float)(t * (1.0/9)). */
static void blur3_replicate(float* m, int w, int h, double* rowbuf) {
    for (int y = 0; y < h; ++y)
        for (int x = 0; x < w; ++x) {
            const int x0 = x > 0 ? x - 1 : 0, x1 = x < w - 1 ? x + 1 : w - 1;
            rowbuf[(size_t)y * w + x] =
                ((double)m[(size_t)y * w + x0] + (double)m[(size_t)y * w + x]) + (double)m[(size_t)y * w + x1];
        }
    for (int y = 0; y < h; ++y) {
        const int y0 = y > 0 ? y - 1 : 0, y1 = y < h - 1 ? y + 1 : h - 1;
        for (int x = 0; x < w; ++x) {
            const double t = (rowbuf[(size_t)y0 * w + x] + rowbuf[(size_t)y * w + x]) + rowbuf[(size_t)y1 * w + x];
            m[(size_t)y * w + x] = (float)(t * (1.0 / 9.0));
        }
    }
}

/* GetGlobalWordWeight, :1600-1602: (float)cv::sum(map), the sum taken in double in raster order */
static float gword_weight_sum(const float* m, size_t n) {
    double s = 0.0;
    for (size_t i = 0; i < n; ++i) s += (double)m[i];
    return (float)s;
}

/* ---- refreshModel(nBaseOccCount, fOccDecrFrac, bForceFGUpdate), :107-429 ---- */
int opawcs_refresh_model(opawcs_t* o, size_t base_occ, float decr, int force) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!(decr >= 0.0f && decr <= 1.0f)) return OSUB_EBADARG;
    const int C = o->C, W = o->W, H = o->H;
    const size_t L = o->L, G = o->G;
    const uint64_t t = o->frame_idx;
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        if (!(force || !o->lastFGdil[px])) continue;
        olword* d = o->lw + m * L;
        size_t colorThr, descThr;
        thresholds(o, px, &colorThr, &descThr);
        /* local decrement */
        if (decr > 0.0f)
            for (size_t i = 0; i < L; ++i)
                if (d[i].valid) d[i].occ -= (uint64_t)(decr * (float)d[i].occ);
        const int x0 = (int)(px % W), y0 = (int)(px / W);
        for (int it = 0; it < 7 * 7 * 2; ++it) {
            /* local resampling */
            int sx, sy;
            sample_pos_7x7(pdraw(o, px), &sx, &sy, x0, y0, LBSP_BORDER, W, H);
            const size_t spx = (size_t)W * sy + sx;
            if (!(force || !o->lastFGdil[spx])) continue;
            const uint8_t* scol = o->lastColor + spx * C;
            const uint16_t* sdesc = o->lastDesc + spx * C;
            int uninit = 0;
            size_t i;
            for (i = 0; i < L; ++i) {
                if (d[i].valid) {
                    const int match = C == 1 ? (absdiff(scol[0], d[i].color[0]) <= colorThr &&
                                                popc16(sdesc[0] ^ d[i].desc[0]) <= descThr)
                                             : (cmixdist3(scol, d[i].color) <= colorThr &&
                                                hdist3(sdesc, d[i].desc) <= descThr);
                    if (match) {
                        d[i].occ += DEFAULT_LWORD_OCC_INCR;
                        d[i].last = t;
                        break;
                    }
                } else {
                    uninit = 1;
                }
            }
            if (i == L) {
                i = L - 1;
                (void)uninit; /* a fresh pool word or the last slot's word: either way slot L-1 gets it */
                for (int c = 0; c < C; ++c) {
                    d[i].color[c] = scol[c];
                    d[i].desc[c] = sdesc[c];
                }
                d[i].occ = base_occ;
                d[i].first = t;
                d[i].last = t;
                d[i].valid = 1;
            }
            while (i > 0 && (!d[i - 1].valid || lword_weight(&d[i], t, o->lword_offset) >
                                                    lword_weight(&d[i - 1], t, o->lword_offset))) {
                const olword tmp = d[i];
                d[i] = d[i - 1];
                d[i - 1] = tmp;
                --i;
            }
        }
        for (size_t i = 1; i < L; ++i) {
            /* local random resampling of the slots still empty */
            if (d[i].valid) continue;
            const size_t ri = (size_t)pdraw(o, px) % i;
            const olword ref = d[ri];
            int off;
            if (C == 1) off = (int)((size_t)pdraw(o, px) % (colorThr + 1)) - (int)colorThr / 2;
            else off = (int)((size_t)pdraw(o, px) % (colorThr / 3 + 1)) - (int)(colorThr / 6);
            for (int c = 0; c < C; ++c) {
                const int v = (int)ref.color[c] + off;
                d[i].color[c] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
                d[i].desc[c] = ref.desc[c];
            }
            const uint64_t occ = (uint64_t)((float)ref.occ * ((float)(L - i) / (float)L));
            d[i].occ = occ > 1 ? occ : 1;
            d[i].first = t;
            d[i].last = t;
            d[i].valid = 1;
        }
    }
    /* global resampling from equally spaced pixels, two passes */
    const size_t gmap = (size_t)o->gw_w * o->gw_h;
    size_t incr = o->npx / G > 1 ? o->npx / G : 1;
    for (int pass = 0; pass < GWORD_DEFAULT_NB_INIT_SAMPL_PASSES; ++pass) {
        for (size_t m = 0; m < o->n_rel; ++m) {
            const size_t px = o->pxlut[m];
            if ((px % incr) != 0) continue;
            if (!(force || !o->lastFGdil[px])) continue;
            const size_t gidx = (size_t)((int)(px / W) / GWORD_LOOKUP_MAPS_DOWNSAMPLE_RATIO) * o->gw_w +
                                (size_t)((int)(px % W) / GWORD_LOOKUP_MAPS_DOWNSAMPLE_RATIO);
            size_t colorThr, descThr;
            thresholds(o, px, &colorThr, &descThr);
            const olword* best = o->lw + m * L;
            const float bestW = lword_weight(best, t, o->lword_offset);
            const unsigned bestBits = C == 1 ? popc16(best->desc[0]) : popc3(best->desc);
            int uninit = 0;
            size_t g;
            for (g = 0; g < G; ++g) {
                const int w = o->gdict[g];
                if (w >= 0) {
                    const int match =
                        C == 1 ? (absdiff(o->gw_color[w][0], best->color[0]) <= colorThr &&
                                  absdiff((int)bestBits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR)
                               : (absdiff((int)bestBits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR &&
                                  cmixdist3(best->color, o->gw_color[w]) <= colorThr);
                    if (match) break;
                } else {
                    uninit = 1;
                }
            }
            if (g == G) {
                g = G - 1;
                const int w = uninit ? o->gnext++ : o->gdict[g];
                for (int c = 0; c < C; ++c) {
                    o->gw_color[w][c] = best->color[c];
                    o->gw_desc[w][c] = best->desc[c];
                }
                o->gw_bits[w] = (uint8_t)bestBits;
                memset(o->gw_map + (size_t)w * gmap, 0, gmap * sizeof(float));
                o->gw_weight[w] = 0.0f;
                o->gdict[g] = w;
            }
            const int w = o->gdict[g];
            float* lw = o->gw_map + (size_t)w * gmap + gidx;
            if (*lw < bestW) {
                o->gw_weight[w] += bestW;
                *lw += bestW;
            }
            while (g > 0 && (o->gdict[g - 1] < 0 || o->gw_weight[o->gdict[g]] > o->gw_weight[o->gdict[g - 1]])) {
                const int tmp = o->gdict[g];
                o->gdict[g] = o->gdict[g - 1];
                o->gdict[g - 1] = tmp;
                --g;
            }
        }
        incr = incr / 3 > 1 ? incr / 3 : 1;
    }
    for (size_t g = 0; g < G; ++g) {
        if (o->gdict[g] >= 0) continue;
        const int w = o->gnext++;
        memset(o->gw_color[w], 0, sizeof(o->gw_color[w]));
        memset(o->gw_desc[w], 0, sizeof(o->gw_desc[w]));
        o->gw_bits[w] = 0;
        memset(o->gw_map + (size_t)w * gmap, 0, gmap * sizeof(float));
        o->gw_weight[w] = 0.0f;
        o->gdict[g] = w;
    }
    /* per-pixel global word sort: one bubble pass on the local map weights */
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const size_t gidx = (size_t)((int)(px / W) / 2) * o->gw_w + (size_t)((int)(px % W) / 2);
        uint8_t* lutp = o->glut + px * G;
        float last = o->gw_map[(size_t)lutp[0] * gmap + gidx];
        for (size_t j = 1; j < G; ++j) {
            const float cur = o->gw_map[(size_t)lutp[j] * gmap + gidx];
            if (cur > last) {
                const uint8_t tmp = lutp[j];
                lutp[j] = lutp[j - 1];
                lutp[j - 1] = tmp;
            } else {
                last = cur;
            }
        }
    }
    (void)H;
    return OSUB_OK;
}

/* ---- initialize, :431-557 ---- */
int opawcs_initialize(opawcs_t* o, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    if (!img || W <= 0 || H <= 0) return OSUB_EBADARG;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED;
    const size_t npx = (size_t)W * H;
    /* IIBackgroundSubtractor::initialize_common, BackgroundSubtractionUtils.cpp:70-155 */
    uint8_t* newroi = (uint8_t*)malloc(npx);
    if (!roi && o->roi && o->W == W && o->H == H) {
        /* no new ROI and the same size: the last validated ROI is reused (:86-87) */
        memcpy(newroi, o->roi, npx);
    } else if (!roi) {
        memset(newroi, 255, npx);
    } else {
        for (size_t i = 0; i < npx; ++i)
            if (roi[i] != 0 && roi[i] != 255) {
                free(newroi);
                return OSUB_EBADARG;
            }
        uint8_t* d = (uint8_t*)malloc(npx);
        uint8_t* t = (uint8_t*)malloc(npx);
        box_minmax(roi, d, t, W, H, LBSP_BORDER, 1);
        /* `Mat / 2` rounds half to even: 255 -> 128 (BackgroundSubtractionUtils.cpp:95) */
        for (size_t i = 0; i < npx; ++i) newroi[i] = roi[i] | (uint8_t)((d[i] + 1) / 2);
        free(d);
        free(t);
    }
    size_t orig = 0;
    for (size_t i = 0; i < npx; ++i) orig += newroi[i] != 0;
    if (orig == 0) {
        free(newroi);
        return OSUB_EBADARG;
    }
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            if (x < LBSP_BORDER || y < LBSP_BORDER || x >= W - LBSP_BORDER || y >= H - LBSP_BORDER)
                newroi[(size_t)y * W + x] = 0;
    size_t fin = 0;
    for (size_t i = 0; i < npx; ++i) fin += newroi[i] != 0;
    if (fin == 0) {
        free(newroi);
        return OSUB_EBADARG;
    }
    pfree_state(o);
    o->W = W;
    o->H = H;
    o->C = C;
    o->npx = npx;
    o->roi = newroi;
    o->orig_roi = orig;
    o->n_rel = fin;
    o->frame_idx = 0;
    o->frames_since_reset = 0;
    o->cooldown = 0;
    o->auto_reset = 1; /* IIBackgroundSubtractor constructor default, BackgroundSubtractionUtils.cpp:67 */
    o->moving_cam = 0;
    o->pxlut = (size_t*)malloc(fin * sizeof(size_t));
    o->model = (size_t*)malloc(npx * sizeof(size_t));
    for (size_t i = 0, m = 0; i < npx; ++i) {
        o->model[i] = newroi[i] ? m : (size_t)-1;
        if (newroi[i]) o->pxlut[m++] = i;
    }
    o->lastColor = (uint8_t*)calloc(npx * C, 1);
    for (size_t i = 0; i < npx; ++i)
        if (newroi[i])
            for (int c = 0; c < C; ++c) o->lastColor[i * C + c] = img[i * C + c];
    /* IBackgroundSubtractorLBSP_::initialize_common, BackgroundSubtractorLBSP.cpp:21-65 */
    o->lastDesc = (uint16_t*)calloc(npx * C, sizeof(uint16_t));
    const float rel = o->p.rel_lbsp_threshold;
    for (int t = 0; t <= 255; ++t)
        o->lut[t] = C == 1 ? sat_u8f(((float)t * rel + (float)o->p.lbsp_threshold_offset) / 3)
                           : sat_u8f((float)t * rel + (float)o->p.lbsp_threshold_offset);
    uint8_t vals[16];
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            if (newroi[i] && x > LBSP_BORDER && y > LBSP_BORDER && x < W - LBSP_BORDER && y < H - LBSP_BORDER)
                for (int c = 0; c < C; ++c) {
                    lbsp_lookup(img, W, C, x, y, c, vals);
                    o->lastDesc[i * C + c] = lbsp_threshold(vals, img[i * C + c], o->lut[img[i * C + c]]);
                }
        }
    /* BackgroundSubtractorPAWCS::initialize */
    o->ds_w = W / FRAMELEVEL_DOWNSAMPLE_RATIO;
    o->ds_h = H / FRAMELEVEL_DOWNSAMPLE_RATIO;
    o->gw_w = W / GWORD_LOOKUP_MAPS_DOWNSAMPLE_RATIO;
    o->gw_h = H / GWORD_LOOKUP_MAPS_DOWNSAMPLE_RATIO;
    const size_t nds = (size_t)o->ds_w * o->ds_h;
    o->ds_roi = (uint8_t*)calloc(nds ? nds : 1, 1);
    if (!nds) { /* the reference's cv::resize to an empty size (:446) throws */
        pfree_state(o);
        return OSUB_EBADARG;
    }
    resize_area_int(newroi, W, H, 1, o->ds_roi, o->ds_w, o->ds_h);
    o->last_nonflat_ratio = 0.0f;
    o->L = o->p.max_words;
    const size_t maxG = o->p.max_words / 2;
    if (orig >= npx / 2 && (int)npx >= DEFAULT_FRAME_AREA) {
        const float f = (float)npx / DEFAULT_FRAME_AREA;
        int raw = (int)floorf(0.5f + f) + o->p.default_median_blur_kernel_size;
        const int cap = o->p.default_median_blur_kernel_size + 4;
        raw = raw < cap ? raw : cap;
        o->median_k = (raw % 2) ? raw : raw - 1;
        o->G = maxG;
        for (size_t i = 0; i < nds; ++i) o->ds_roi[i] |= 127;
    } else {
        const float f = (float)orig / DEFAULT_FRAME_AREA;
        int raw = (int)floorf(0.5f + (float)o->p.default_median_blur_kernel_size * f * 2) +
                  (o->p.default_median_blur_kernel_size - 4);
        raw = raw < o->p.default_median_blur_kernel_size ? raw : o->p.default_median_blur_kernel_size;
        o->median_k = (raw % 2) ? raw : raw - 1;
        const float g = (float)maxG * f;
        const size_t gg = (size_t)pow((double)g, 2) + 1;
        o->G = gg < maxG ? gg : maxG;
    }
    if (C == 1) {
        o->L = o->L / 2 > 1 ? o->L / 2 : 1;
        o->G = o->G / 2 > 1 ? o->G / 2 : 1;
    }
    o->ds_roi_count = 0;
    for (size_t i = 0; i < nds; ++i) o->ds_roi_count += o->ds_roi[i] != 0;
    o->lword_offset = DEFAULT_LWORD_WEIGHT_OFFSET;
    float** fmaps[] = {&o->R, &o->V, &o->T, &o->DminLT, &o->DminST, &o->RawLT, &o->RawST, &o->FinLT, &o->FinST};
    for (size_t m = 0; m < sizeof(fmaps) / sizeof(fmaps[0]); ++m) *fmaps[m] = (float*)calloc(npx, sizeof(float));
    for (size_t i = 0; i < npx; ++i) {
        o->T[i] = FEEDBACK_T_LOWER;
        o->R[i] = 2.0f;
        o->V[i] = FEEDBACK_V_INCR * 10;
    }
    const size_t ndsC = nds * (size_t)C;
    o->dsLT = (float*)calloc(ndsC > 0 ? ndsC : 1, sizeof(float));
    o->dsST = (float*)calloc(ndsC > 0 ? ndsC : 1, sizeof(float));
    o->dsframe = (uint8_t*)calloc(ndsC > 0 ? ndsC : 1, 1);
    uint8_t** bmaps[] = {&o->illum,    &o->unstable,  &o->blinks, &o->lastRawFG, &o->lastFG, &o->lastFGdil,
                         &o->lastFGdilInv, &o->lastRawBlink, &o->currBlink, &o->preflood, &o->holes, &o->tmp8,
                         &o->tmp8b,    &o->visited,   &o->raw};
    for (size_t m = 0; m < sizeof(bmaps) / sizeof(bmaps[0]); ++m) *bmaps[m] = (uint8_t*)calloc(npx, 1);
    o->colcnt = (uint16_t*)calloc(npx, sizeof(uint16_t));
    o->bfs = (int*)malloc(npx * sizeof(int));
    o->lw = (olword*)calloc(fin * o->L, sizeof(olword));
    const size_t gmap = (size_t)o->gw_w * o->gw_h;
    o->gw_map = (float*)calloc(o->G * (gmap ? gmap : 1), sizeof(float));
    for (size_t g = 0; g < 64; ++g) o->gdict[g] = -1;
    o->gnext = 0;
    o->glut = (uint8_t*)calloc(npx * o->G, 1);
    for (size_t i = 0; i < npx; ++i)
        if (newroi[i])
            for (size_t g = 0; g < o->G; ++g) o->glut[i * o->G + g] = (uint8_t)g;
    o->kctr = (uint32_t*)calloc(npx, sizeof(uint32_t));
    o->initialized = 1;
    reset_draws(o);
    opawcs_refresh_model(o, 1, 0.0f, 0);
    return OSUB_OK;
}

/* ---- apply, :559-1561 ---- */
int opawcs_apply(opawcs_t* o, const uint8_t* img, uint8_t* mask, double lr) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const int W = o->W, H = o->H, C = o->C;
    const size_t L = o->L, G = o->G, npx = o->npx;
    uint8_t* raw = o->raw;
    memset(raw, 0, npx);
    reset_draws(o);
    const int boot = ++o->frame_idx <= DEFAULT_BOOTSTRAP_WIN_SIZE;
    const uint64_t t = o->frame_idx;
    const size_t nLT = boot ? o->p.samples_for_moving_avgs / 2 : o->p.samples_for_moving_avgs;
    const size_t nST = nLT / 4;
    const float fLT = 1.0f / (float)(t < nLT ? t : nLT);
    const float fST = 1.0f / (float)(t < nST ? t : nST);
    const size_t gwRate = boot ? DEFAULT_RESAMPLING_RATE / 2 : DEFAULT_RESAMPLING_RATE;
    const size_t gmap = (size_t)o->gw_w * o->gw_h;
    const float initW = 1.0f / (float)o->lword_offset; /* DEFAULT_LWORD_INIT_WEIGHT */
    const size_t colorRange = C == 1 ? 255 : 765, descRange = C == 1 ? 16 : 48;
    const unsigned flatBits = C == 1 ? FLAT_REGION_BIT_COUNT : FLAT_REGION_BIT_COUNT * 2;
    size_t nFlat = 0;
    uint8_t vals[3][16];
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const int x = (int)(px % W), y = (int)(px / W);
        const size_t gidx = (size_t)(y / 2) * o->gw_w + (size_t)(x / 2);
        const uint8_t* col = img + px * C;
        olword* d = o->lw + m * L;
        size_t minColor = colorRange, minDesc = descRange;
        float* R = &o->R[px];
        float* V = &o->V[px];
        float* T = &o->T[px];
        float* dLT = &o->DminLT[px];
        float* dST = &o->DminST[px];
        float* rLT = &o->RawLT[px];
        float* rST = &o->RawST[px];
        const float bestW = lword_weight(&d[0], t, o->lword_offset);
        const float thrW = bestW / (*R * 2);
        uint8_t* unstable = &o->unstable[px];
        uint8_t* illum = &o->illum[px];
        const int border = o->roi[px] < 255;
        uint16_t desc[3] = {0, 0, 0};
        for (int c = 0; c < C; ++c) {
            lbsp_lookup(img, W, C, x, y, c, vals[c]);
            desc[c] = lbsp_threshold(vals[c], col[c], o->lut[col[c]]);
        }
        const unsigned bits = C == 1 ? popc16(desc[0]) : popc3(desc);
        const int flat = bits < flatBits;
        if (flat) ++nFlat;
        const uint64_t incr = (uint64_t)(DEFAULT_LWORD_OCC_INCR + o->cooldown) << (int)(flat || boot);
        uint64_t rate;
        if (isinf(lr)) rate = UINT64_MAX;
        else if (lr > 0) rate = (uint64_t)ceil(lr);
        else if (flat) rate = (uint64_t)ceilf(*T + FEEDBACK_T_LOWER) / 2;
        else rate = (uint64_t)ceilf(*T);
        size_t colorThr, descThr;
        thresholds(o, px, &colorThr, &descThr);
        size_t i = 0;
        float sumW = 0.0f, lastW = FLT_MAX;
        while (i < L && sumW < thrW) {
            olword* w = &d[i];
            const float curW = lword_weight(w, t, o->lword_offset);
            o->st_words_scanned++;
            size_t colorDist, colorL1, intraDist, interDist;
            if (C == 1) {
                colorDist = colorL1 = absdiff(col[0], w->color[0]);
                intraDist = popc16(desc[0] ^ w->desc[0]);
                const uint16_t inter = lbsp_threshold(vals[0], w->color[0], o->lut[w->color[0]]);
                interDist = popc16(inter ^ w->desc[0]);
            } else {
                colorL1 = l1dist3(col, w->color);
                colorDist = colorL1 / 2 + cdist3(col, w->color) * 4;
                intraDist = hdist3(desc, w->desc);
                uint16_t inter[3];
                for (int c = 0; c < 3; ++c) inter[c] = lbsp_threshold(vals[c], w->color[c], o->lut[w->color[c]]);
                interDist = hdist3(inter, w->desc);
            }
            const size_t descDist = (intraDist + interDist) / 2;
            if ((!*unstable || flat || border) && colorDist <= colorThr && colorL1 >= colorThr / 2 &&
                intraDist <= descThr / 2) {
                const uint64_t mod = *illum ? (rate / 2 + 1) : rate;
                if ((uint64_t)pdraw(o, px) % mod == 0) {
                    /* illumination update */
                    for (int c = 0; c < C; ++c) {
                        w->color[c] = col[c];
                        w->desc[c] = desc[c];
                    }
                    o->illum[px - 1] = 1 & o->roi[px - 1];
                    o->illum[px + 1] = 1 & o->roi[px + 1];
                    o->illum[px] = 2;
                }
            }
            if (descDist <= descThr && colorDist <= colorThr) {
                sumW += curW;
                w->last = t;
                if ((!o->lastFG[px] || o->moving_cam) && curW < DEFAULT_LWORD_MAX_WEIGHT) w->occ += incr;
                minColor = minColor < colorDist ? minColor : colorDist;
                minDesc = minDesc < descDist ? minDesc : descDist;
            }
            if (curW > lastW) {
                const olword tmp = d[i];
                d[i] = d[i - 1];
                d[i - 1] = tmp;
            } else {
                lastW = curW;
            }
            ++i;
        }
        while (i < L) {
            const float curW = lword_weight(&d[i], t, o->lword_offset);
            if (curW > lastW) {
                const olword tmp = d[i];
                d[i] = d[i - 1];
                d[i - 1] = tmp;
            } else {
                lastW = curW;
            }
            ++i;
        }
        uint8_t* segm = &raw[px];
        const uint8_t* lutp = o->glut + px * G;
        if (sumW >= thrW || border) {
            /* background */
            const float nd = maxf_std((float)minColor / (float)colorRange, (float)minDesc / (float)descRange);
            *dLT = *dLT * (1.0f - fLT) + nd * fLT;
            *dST = *dST * (1.0f - fST) + nd * fST;
            *rLT = *rLT * (1.0f - fLT);
            *rST = *rST * (1.0f - fST);
            if ((uint64_t)pdraw(o, px) % rate == 0) {
                o->st_gdict_events++;
                size_t g;
                int w = -1;
                for (g = 0; g < G; ++g) {
                    w = lutp[g];
                    const int match =
                        C == 1 ? (absdiff(o->gw_color[w][0], col[0]) <= colorThr &&
                                  absdiff((int)bits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR)
                               : (absdiff((int)bits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR &&
                                  cmixdist3(col, o->gw_color[w]) <= colorThr);
                    if (match) break;
                }
                if (g != G || (uint64_t)pdraw(o, px) % (rate * 2) == 0) {
                    if (g == G) {
                        w = o->gdict[G - 1];
                        for (int c = 0; c < C; ++c) {
                            o->gw_color[w][c] = col[c];
                            o->gw_desc[w][c] = desc[c];
                        }
                        o->gw_bits[w] = (uint8_t)bits;
                        memset(o->gw_map + (size_t)w * gmap, 0, gmap * sizeof(float));
                        o->gw_weight[w] = 0.0f;
                    }
                    float* lwp = o->gw_map + (size_t)w * gmap + gidx;
                    if (*lwp < sumW) {
                        o->gw_weight[w] += sumW;
                        *lwp += sumW;
                    }
                }
            }
        } else {
            /* foreground */
            const float nd = maxf_std(maxf_std((float)minColor / (float)colorRange, (float)minDesc / (float)descRange),
                                      (thrW - sumW) / thrW);
            *dLT = *dLT * (1.0f - fLT) + nd * fLT;
            *dST = *dST * (1.0f - fST) + nd * fST;
            *rLT = *rLT * (1.0f - fLT) + fLT;
            *rST = *rST * (1.0f - fST) + fST;
            if (flat || (uint64_t)pdraw(o, px) % rate == 0) {
                size_t g;
                int w = -1;
                for (g = 0; g < G; ++g) {
                    w = lutp[g];
                    const int match =
                        C == 1 ? (absdiff(o->gw_color[w][0], col[0]) <= colorThr &&
                                  absdiff((int)bits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR)
                               : (absdiff((int)bits, o->gw_bits[w]) <= descThr / GWORD_DESC_THRES_BITS_MATCH_FACTOR &&
                                  cmixdist3(col, o->gw_color[w]) <= colorThr);
                    if (match) break;
                }
                if (g == G) {
                    *segm = 255;
                } else {
                    const float gl = o->gw_map[(size_t)w * gmap + gidx];
                    if (sumW + gl / (float)(flat ? 2 : 4) < thrW) *segm = 255;
                }
            } else {
                *segm = 255;
            }
            if (sumW < initW) {
                olword* nw = &d[L - 1];
                for (int c = 0; c < C; ++c) {
                    nw->color[c] = col[c];
                    nw->desc[c] = desc[c];
                }
                nw->occ = incr;
                nw->first = t;
                nw->last = t;
            }
        }
        /* neighbour update */
        if ((!*segm && (uint64_t)pdraw(o, px) % rate == 0) || border || o->moving_cam) {
            o->st_nb_updates++;
            int nx, ny;
            neighbor_pos(pdraw(o, px), !(flat || border || o->moving_cam), &nx, &ny, x, y, LBSP_BORDER, W, H);
            const size_t q = (size_t)W * ny + nx;
            if (o->roi[q]) {
                olword* nd = o->lw + o->model[q] * L;
                size_t j = 0;
                float nsum = 0.0f;
                while (j < L && nsum < thrW) {
                    olword copy = nd[j];
                    /* one channel: the reference updates a copy of the word (:838); three: the word */
                    olword* nw = C == 1 ? &copy : &nd[j];
                    size_t ncolorDist, nintra, ncd = 0, ncolorL1;
                    unsigned nbits;
                    if (C == 1) {
                        ncolorDist = ncolorL1 = absdiff(col[0], nw->color[0]);
                        nintra = popc16(desc[0] ^ nw->desc[0]);
                        nbits = popc16(nw->desc[0]);
                    } else {
                        ncolorL1 = l1dist3(col, nw->color);
                        ncd = cdist3(col, nw->color);
                        ncolorDist = ncolorL1 / 2 + ncd * 4;
                        nintra = hdist3(desc, nw->desc);
                        nbits = popc3(nw->desc);
                    }
                    const int nflat = nbits < flatBits;
                    const uint64_t nincr = nflat ? incr * 2 : incr;
                    if (ncolorDist <= colorThr && nintra <= descThr) {
                        const float nwW = lword_weight(nw, t, o->lword_offset);
                        nsum += nwW;
                        nw->last = t;
                        if (nwW < DEFAULT_LWORD_MAX_WEIGHT) nw->occ += nincr;
                    } else if (!raw[q] && flat && (boot || (uint64_t)pdraw(o, px) % rate == 0)) {
                        const uint16_t* nlast = o->lastDesc + q * C;
                        const size_t nlastDist = C == 1 ? popc16(desc[0] ^ nlast[0]) : hdist3(desc, nlast);
                        if (ncolorDist <= colorThr && nlastDist <= descThr / 2) {
                            const float nwW = lword_weight(nw, t, o->lword_offset);
                            nsum += nwW;
                            nw->last = t;
                            if (nwW < DEFAULT_LWORD_MAX_WEIGHT) nw->occ += nincr;
                            for (int c = 0; c < C; ++c) nw->desc[c] = desc[c];
                        } else if (C == 3) {
                            const int nlastFlat = popc3(nlast) < flatBits;
                            if (nlastFlat && flat && nlastDist + nintra <= descThr && ncd <= colorThr / 4) {
                                const float nwW = lword_weight(nw, t, o->lword_offset);
                                nsum += nwW;
                                nw->last = t;
                                if (nwW < DEFAULT_LWORD_MAX_WEIGHT) nw->occ += nincr;
                                for (int c = 0; c < 3; ++c) nw->color[c] = col[c];
                            }
                        }
                    }
                    ++j;
                }
                if (nsum < initW) {
                    olword* nw = &nd[L - 1];
                    for (int c = 0; c < C; ++c) {
                        nw->color[c] = col[c];
                        nw->desc[c] = desc[c];
                    }
                    nw->occ = incr;
                    nw->first = t;
                    nw->last = t;
                }
            }
        }
        if (*illum) *illum -= 1;
        /* feedback adjustments */
        *unstable = *R > UNSTABLE_REG_RDIST_MIN || (*rLT - o->FinLT[px]) > UNSTABLE_REG_RATIO_MIN ||
                    (*rST - o->FinST[px]) > UNSTABLE_REG_RATIO_MIN;
        const float dmin = minf_std(*dLT, *dST), dmax = maxf_std(*dLT, *dST);
        if (o->lastFG[px] || (dmin < UNSTABLE_REG_RATIO_MIN && *segm))
            *T = minf_std(*T + FEEDBACK_T_INCR / (dmax * *V), FEEDBACK_T_UPPER);
        else
            *T = maxf_std(*T - FEEDBACK_T_DECR * *V / dmax, FEEDBACK_T_LOWER);
        if (dmax > UNSTABLE_REG_RATIO_MIN && o->blinks[px])
            *V += boot ? FEEDBACK_V_INCR * 2 : FEEDBACK_V_INCR;
        else
            *V = maxf_std(*V - FEEDBACK_V_DECR * ((boot || flat) ? 2.0f : o->lastFG[px] ? 0.5f : 1.0f), FEEDBACK_V_DECR);
        const float base = 1.0f + dmin * 2;
        if ((double)*R < (double)base * (double)base) /* std::pow(float,int) promotes to double */
            *R += FEEDBACK_R_VAR * (*V - FEEDBACK_V_DECR);
        else
            *R = maxf_std(*R - FEEDBACK_R_VAR / *V, 1.0f);
        for (int c = 0; c < C; ++c) {
            o->lastDesc[px * C + c] = desc[c];
            o->lastColor[px * C + c] = col[c];
        }
    }
    /* global words, :1300-1334 */
    const int recalc = !(t % (gwRate << 5));
    const int update = !(t % gwRate);
    if (update) {
        /* cv::resize(lastFGdilInv, ds, (W/2, H/2), INTER_NEAREST): source x = floor(dx * W/dW) */
        const double ifx = 1.0 / ((double)o->gw_w / W), ify = 1.0 / ((double)o->gw_h / H);
        for (int yy = 0; yy < o->gw_h; ++yy) {
            int sy = (int)floor(yy * ify);
            sy = sy < H - 1 ? sy : H - 1;
            for (int xx = 0; xx < o->gw_w; ++xx) {
                int sx = (int)floor(xx * ifx);
                sx = sx < W - 1 ? sx : W - 1;
                o->tmp8[(size_t)yy * o->gw_w + xx] = o->lastFGdilInv[(size_t)sy * W + sx];
            }
        }
    }
    double* rowbuf = update ? (double*)malloc((gmap ? gmap : 1) * sizeof(double)) : NULL;
    for (size_t g = 0; g < G; ++g) {
        const int w = o->gdict[g];
        float* mp = o->gw_map + (size_t)w * gmap;
        if (recalc && o->gw_weight[w] > 0.0f) {
            o->gw_weight[w] = gword_weight_sum(mp, gmap);
            if (o->gw_weight[w] < 1.0f) {
                o->gw_weight[w] = 0.0f;
                memset(mp, 0, gmap * sizeof(float));
            }
        }
        if (update && o->gw_weight[w] > 0.0f) {
            /* cv::accumulateProduct(map, -0.1, map, mask): map += map * -0.1f where the mask is set */
            for (size_t k = 0; k < gmap; ++k)
                if (o->tmp8[k]) {
                    const float prod = mp[k] * -0.1f;
                    mp[k] = mp[k] + prod;
                }
            o->gw_weight[w] *= 0.9f;
            blur3_replicate(mp, o->gw_w, o->gw_h, rowbuf);
        }
        if (g > 0 && o->gw_weight[o->gdict[g]] > o->gw_weight[o->gdict[g - 1]]) {
            const int tmp = o->gdict[g];
            o->gdict[g] = o->gdict[g - 1];
            o->gdict[g - 1] = tmp;
        }
    }
    free(rowbuf);
    if (update) {
        for (size_t m = 0; m < o->n_rel; ++m) {
            const size_t px = o->pxlut[m];
            const size_t gidx = (size_t)((int)(px / W) / 2) * o->gw_w + (size_t)((int)(px % W) / 2);
            uint8_t* lutp = o->glut + px * G;
            float last = o->gw_map[(size_t)lutp[0] * gmap + gidx];
            for (size_t j = 1; j < G; ++j) {
                const float cur = o->gw_map[(size_t)lutp[j] * gmap + gidx];
                if (cur > last) {
                    const uint8_t tmp = lutp[j];
                    lutp[j] = lutp[j - 1];
                    lutp[j - 1] = tmp;
                } else {
                    last = cur;
                }
            }
        }
    }
    /* post-processing, :1443-1461 */
    for (size_t i = 0; i < npx; ++i) {
        o->currBlink[i] = raw[i] ^ o->lastRawFG[i];
        o->blinks[i] = o->currBlink[i] | o->lastRawBlink[i];
        o->lastRawBlink[i] = o->currBlink[i];
        o->lastRawFG[i] = raw[i];
    }
    /* morphologyEx(CLOSE, 3x3): dilate then erode, clipped windows */
    box_minmax(raw, o->tmp8b, o->tmp8, W, H, 1, 1);
    box_minmax(o->tmp8b, o->preflood, o->tmp8, W, H, 1, 0);
    pflood_holes(o, o->preflood, o->holes);
    box_minmax(o->preflood, o->tmp8b, o->tmp8, W, H, 3, 0);
    for (size_t i = 0; i < npx; ++i) raw[i] = raw[i] | o->holes[i] | o->tmp8b[i];
    median_binary(raw, o->lastFG, o->colcnt, W, H, o->median_k);
    box_minmax(o->lastFG, o->lastFGdil, o->tmp8, W, H, 3, 1);
    for (size_t i = 0; i < npx; ++i) {
        o->blinks[i] &= o->lastFGdilInv[i];
        o->lastFGdilInv[i] = (uint8_t)~o->lastFGdil[i];
        o->blinks[i] &= o->lastFGdilInv[i];
    }
    if (mask) memcpy(mask, o->lastFG, npx);
    add_weighted_mask(o->FinLT, o->lastFG, npx, (double)(1.0f - fLT), (1.0 / 255) * fLT);
    add_weighted_mask(o->FinST, o->lastFG, npx, (double)(1.0f - fST), (1.0 / 255) * fST);
    const float nonflat = (float)(o->n_rel - nFlat) / (float)o->n_rel;
    if (nonflat < LBSPDESC_RATIO_MIN && o->last_nonflat_ratio < LBSPDESC_RATIO_MIN) {
        for (int k = 0; k <= 255; ++k)
            if (o->lut[k] > sat_u8f(((float)o->p.lbsp_threshold_offset + (float)k * o->p.rel_lbsp_threshold) / 4))
                --o->lut[k];
    } else if (nonflat > LBSPDESC_RATIO_MAX && o->last_nonflat_ratio > LBSPDESC_RATIO_MAX) {
        for (int k = 0; k <= 255; ++k)
            if (o->lut[k] < sat_u8f((float)o->p.lbsp_threshold_offset + 255 * o->p.rel_lbsp_threshold)) ++o->lut[k];
    }
    o->last_nonflat_ratio = nonflat;
    /* automatic model reset, :1462-1516 */
    const size_t nds = (size_t)o->ds_w * o->ds_h;
    if (nds && resize_area_int(img, W, H, C, o->dsframe, o->ds_w, o->ds_h)) {
        accumulate_weighted(o->dsframe, o->dsLT, nds * C, fLT);
        accumulate_weighted(o->dsframe, o->dsST, nds * C, fST);
        float l1 = 0.0f;
        for (size_t k = 0; k < nds; ++k)
            if (o->ds_roi[k]) {
                float e = 0.0f;
                for (int c = 0; c < C; ++c) e += fabsf(o->dsLT[k * C + c] - o->dsST[k * C + c]);
                l1 += e;
            }
        const float ratio = l1 / (float)o->ds_roi_count;
        if (!o->auto_reset && ratio >= FRAMELEVEL_MIN_L1DIST_THRES * 2) o->auto_reset = 1;
        if (o->auto_reset || o->moving_cam) {
            if ((t % DEFAULT_BOOTSTRAP_WIN_SIZE) == 0) {
                /* background image vs the long-term mean of the down-sampled frames */
                uint8_t* bg = (uint8_t*)malloc(npx * C);
                uint8_t* dsbg = (uint8_t*)malloc(nds * C);
                opawcs_get_background(o, bg);
                resize_area_int(bg, W, H, C, dsbg, o->ds_w, o->ds_h);
                float ml1 = 0.0f, mcd = 0.0f;
                for (size_t k = 0; k < nds; ++k)
                    if (o->ds_roi[k] == 255) {
                        float e = 0.0f;
                        for (int c = 0; c < C; ++c) e += fabsf(o->dsLT[k * C + c] - (float)dsbg[k * C + c]);
                        ml1 += e;
                        if (C == 3) {
                            /* lv::cdist<3> for floats, math.hpp:499-527 */
                            const float* a = o->dsLT + k * 3;
                            float b[3] = {(float)dsbg[k * 3], (float)dsbg[k * 3 + 1], (float)dsbg[k * 3 + 2]};
                            int nonconst = 0, nonnull = a[0] != b[0];
                            for (int c = 1; c < 3; ++c) {
                                nonconst |= (a[c] != a[c - 1]) || (b[c] != b[c - 1]);
                                nonnull |= a[c] != b[c];
                            }
                            float cd = 0.0f;
                            if (nonconst && nonnull) {
                                float cs = 0, bs = 0, mx = 0;
                                for (int c = 0; c < 3; ++c) {
                                    cs += a[c] * a[c];
                                    bs += b[c] * b[c];
                                    mx += a[c] * b[c];
                                }
                                bs += FLT_EPSILON;
                                if (!(cs <= (mx * mx) / bs)) cd = sqrtf(cs - (mx * mx) / bs);
                            }
                            mcd += cd;
                        }
                    }
                free(bg);
                free(dsbg);
                const float mr = ml1 / (float)o->ds_roi_count;
                const float cr = C == 1 ? 0.0f : mcd / (float)o->ds_roi_count;
                if (o->moving_cam && mr < FRAMELEVEL_MIN_L1DIST_THRES / 4 && cr < FRAMELEVEL_MIN_CDIST_THRES / 4) {
                    o->lword_offset = DEFAULT_LWORD_WEIGHT_OFFSET;
                    o->moving_cam = 0;
                    opawcs_refresh_model(o, 1, 1.0f, 1);
                } else if (boot && !o->moving_cam &&
                           (mr >= FRAMELEVEL_MIN_L1DIST_THRES || cr >= FRAMELEVEL_MIN_CDIST_THRES)) {
                    o->lword_offset = 5;
                    o->moving_cam = 1;
                    opawcs_refresh_model(o, 1, 1.0f, 1);
                }
            }
            if (o->frames_since_reset > DEFAULT_BOOTSTRAP_WIN_SIZE * 2) {
                o->auto_reset = 0;
            } else if (ratio >= FRAMELEVEL_MIN_L1DIST_THRES && o->cooldown == 0) {
                o->frames_since_reset = 0;
                opawcs_refresh_model(o, o->lword_offset / 8, 0.0f, 1);
                o->cooldown = nST;
                for (size_t k = 0; k < npx; ++k) o->T[k] = 1.0f;
            } else if (!boot) {
                ++o->frames_since_reset;
            }
        }
    }
    if (o->cooldown > 0) --o->cooldown;
    return OSUB_OK;
}

/* getBackgroundImage, :1535-1567: weight-averaged word colours, convertTo(CV_8U) */
/* setROI, BackgroundSubtractionUtils.cpp:38-48, with validateROI :28-36 */
int opawcs_set_roi(opawcs_t* o, const uint8_t* roi, int W, int H) {
    if (!roi || W <= 0 || H <= 0) return OSUB_EBADARG;
    const size_t npx = (size_t)W * H;
    uint8_t* r = (uint8_t*)malloc(npx);
    size_t nz = 0;
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t i = (size_t)y * W + x;
            r[i] = (x < LBSP_BORDER || y < LBSP_BORDER || x >= W - LBSP_BORDER || y >= H - LBSP_BORDER) ? 0 : roi[i];
            nz += r[i] != 0;
        }
    if (nz == 0) {
        free(r);
        return OSUB_EBADARG;
    }
    if (o->initialized) {
        if (W != o->W || H != o->H) {
            free(r);
            return OSUB_EBADARG;
        }
        uint8_t* bg = (uint8_t*)malloc(npx * (size_t)o->C);
        opawcs_get_background(o, bg);
        const int st = opawcs_initialize(o, bg, W, H, o->C, r);
        free(bg);
        free(r);
        return st;
    }
    free(o->roi);
    o->roi = r;
    o->W = W;
    o->H = H;
    return OSUB_OK;
}

int opawcs_get_background(const opawcs_t* o, uint8_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const int C = o->C;
    memset(out, 0, o->npx * C);
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const olword* d = o->lw + m * o->L;
        float tw = 0.0f, tc[3] = {0.0f, 0.0f, 0.0f};
        for (size_t i = 0; i < o->L; ++i) {
            const float w = lword_weight(&d[i], o->frame_idx, o->lword_offset);
            for (int c = 0; c < C; ++c) tc[c] += (float)d[i].color[c] * w;
            tw += w;
        }
        for (int c = 0; c < C; ++c) out[px * C + c] = sat_u8f(tc[c] / tw);
    }
    return OSUB_OK;
}

/* getBackgroundDescriptorsImage, :1569-1594: weight-averaged word descriptors, convertTo(CV_16U) */
int opawcs_get_background_descriptors(const opawcs_t* o, uint16_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const int C = o->C;
    memset(out, 0, o->npx * C * sizeof(uint16_t));
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const olword* d = o->lw + m * o->L;
        float tw = 0.0f, td[3] = {0.0f, 0.0f, 0.0f};
        for (size_t i = 0; i < o->L; ++i) {
            const float w = lword_weight(&d[i], o->frame_idx, o->lword_offset);
            for (int c = 0; c < C; ++c) td[c] += (float)d[i].desc[c] * w;
            tw += w;
        }
        for (int c = 0; c < C; ++c) out[px * C + c] = sat_u16f(td[c] / tw);
    }
    return OSUB_OK;
}

/* model state for parity checks; word planes are exported slot-major per model index */
int opawcs_export(const opawcs_t* o, int which, void* out, size_t bytes) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t npx = o->npx, nw = o->n_rel * o->L, C = (size_t)o->C, gmap = (size_t)o->gw_w * o->gw_h;
    const size_t nds = (size_t)o->ds_w * o->ds_h * C;
    size_t need = 0;
    const void* src = NULL;
    switch (which) {
    case OPAWCS_MAP_R: src = o->R; need = npx * 4; break;
    case OPAWCS_MAP_V: src = o->V; need = npx * 4; break;
    case OPAWCS_MAP_T: src = o->T; need = npx * 4; break;
    case OPAWCS_MAP_DMIN_LT: src = o->DminLT; need = npx * 4; break;
    case OPAWCS_MAP_DMIN_ST: src = o->DminST; need = npx * 4; break;
    case OPAWCS_MAP_RAW_LT: src = o->RawLT; need = npx * 4; break;
    case OPAWCS_MAP_RAW_ST: src = o->RawST; need = npx * 4; break;
    case OPAWCS_MAP_FIN_LT: src = o->FinLT; need = npx * 4; break;
    case OPAWCS_MAP_FIN_ST: src = o->FinST; need = npx * 4; break;
    case OPAWCS_MAP_ILLUM: src = o->illum; need = npx; break;
    case OPAWCS_MAP_UNSTABLE: src = o->unstable; need = npx; break;
    case OPAWCS_MAP_BLINKS: src = o->blinks; need = npx; break;
    case OPAWCS_MAP_LAST_RAW_FG: src = o->lastRawFG; need = npx; break;
    case OPAWCS_MAP_LAST_FG: src = o->lastFG; need = npx; break;
    case OPAWCS_MAP_LAST_FG_DIL: src = o->lastFGdil; need = npx; break;
    case OPAWCS_MAP_LAST_RAW_BLINK: src = o->lastRawBlink; need = npx; break;
    case OPAWCS_MAP_ROI: src = o->roi; need = npx; break;
    case OPAWCS_MAP_LAST_COLOR: src = o->lastColor; need = npx * C; break;
    case OPAWCS_MAP_LAST_DESC: src = o->lastDesc; need = npx * C * 2; break;
    case OPAWCS_MAP_DS_LT: src = o->dsLT; need = nds * 4; break;
    case OPAWCS_MAP_DS_ST: src = o->dsST; need = nds * 4; break;
    case OPAWCS_MAP_LUT: src = o->lut; need = 256; break;
    case OPAWCS_MAP_GW_MAP: src = o->gw_map; need = o->G * gmap * 4; break;
    case OPAWCS_MAP_GLUT: {
        need = npx * o->G;
        if (!out || bytes < need) return OSUB_EBADARG;
        memcpy(out, o->glut, need);
        return OSUB_OK;
    }
    case OPAWCS_MAP_GW: {
        /* per pool word: colour[3] u8, pad u8, desc[3] u16, bits u8, pad u8, weight f32, dict slot i32 */
        need = o->G * 20;
        if (!out || bytes < need) return OSUB_EBADARG;
        uint8_t* b = (uint8_t*)out;
        memset(b, 0, need);
        for (size_t w = 0; w < o->G; ++w) {
            uint8_t* r = b + w * 20;
            memcpy(r, o->gw_color[w], 3);
            memcpy(r + 4, o->gw_desc[w], 6);
            r[10] = o->gw_bits[w];
            memcpy(r + 12, &o->gw_weight[w], 4);
            int32_t slot = -1;
            for (size_t g = 0; g < o->G; ++g)
                if (o->gdict[g] == (int)w) slot = (int32_t)g;
            memcpy(r + 16, &slot, 4);
        }
        return OSUB_OK;
    }
    case OPAWCS_MAP_LW_COLOR:
    case OPAWCS_MAP_LW_DESC:
    case OPAWCS_MAP_LW_OCC:
    case OPAWCS_MAP_LW_FIRST:
    case OPAWCS_MAP_LW_LAST: {
        const size_t es = which == OPAWCS_MAP_LW_COLOR ? C : which == OPAWCS_MAP_LW_DESC ? 2 * C : 8;
        need = nw * es;
        if (!out || bytes < need) return OSUB_EBADARG;
        for (size_t k = 0; k < nw; ++k) {
            const olword* w = o->lw + k;
            uint8_t* r = (uint8_t*)out + k * es;
            if (which == OPAWCS_MAP_LW_COLOR) memcpy(r, w->color, C);
            else if (which == OPAWCS_MAP_LW_DESC) memcpy(r, w->desc, 2 * C);
            else if (which == OPAWCS_MAP_LW_OCC) memcpy(r, &w->occ, 8);
            else if (which == OPAWCS_MAP_LW_FIRST) memcpy(r, &w->first, 8);
            else memcpy(r, &w->last, 8);
        }
        return OSUB_OK;
    }
    default: return OSUB_EBADARG;
    }
    if (!out || bytes < need) return OSUB_EBADARG;
    memcpy(out, src, need);
    return OSUB_OK;
}

size_t opawcs_export_bytes(const opawcs_t* o, int which) {
    if (!o->initialized) return 0;
    const size_t npx = o->npx, nw = o->n_rel * o->L, C = (size_t)o->C, gmap = (size_t)o->gw_w * o->gw_h;
    const size_t nds = (size_t)o->ds_w * o->ds_h * C;
    switch (which) {
    case OPAWCS_MAP_R: case OPAWCS_MAP_V: case OPAWCS_MAP_T: case OPAWCS_MAP_DMIN_LT: case OPAWCS_MAP_DMIN_ST:
    case OPAWCS_MAP_RAW_LT: case OPAWCS_MAP_RAW_ST: case OPAWCS_MAP_FIN_LT: case OPAWCS_MAP_FIN_ST: return npx * 4;
    case OPAWCS_MAP_ILLUM: case OPAWCS_MAP_UNSTABLE: case OPAWCS_MAP_BLINKS: case OPAWCS_MAP_LAST_RAW_FG:
    case OPAWCS_MAP_LAST_FG: case OPAWCS_MAP_LAST_FG_DIL: case OPAWCS_MAP_LAST_RAW_BLINK: case OPAWCS_MAP_ROI:
        return npx;
    case OPAWCS_MAP_LAST_COLOR: return npx * C;
    case OPAWCS_MAP_LAST_DESC: return npx * C * 2;
    case OPAWCS_MAP_DS_LT: case OPAWCS_MAP_DS_ST: return nds * 4;
    case OPAWCS_MAP_LUT: return 256;
    case OPAWCS_MAP_GW_MAP: return o->G * gmap * 4;
    case OPAWCS_MAP_GLUT: return npx * o->G;
    case OPAWCS_MAP_GW: return o->G * 20;
    case OPAWCS_MAP_LW_COLOR: return nw * C;
    case OPAWCS_MAP_LW_DESC: return nw * C * 2;
    case OPAWCS_MAP_LW_OCC: case OPAWCS_MAP_LW_FIRST: case OPAWCS_MAP_LW_LAST: return nw * 8;
    default: return 0;
    }
}

void opawcs_get_scalars(const opawcs_t* o, opawcs_scalars* s) {
    memset(s, 0, sizeof(*s));
    s->frame_idx = o->frame_idx;
    s->frames_since_last_reset = o->frames_since_reset;
    s->model_reset_cooldown = o->cooldown;
    s->lword_weight_offset = o->lword_offset;
    s->auto_model_reset_enabled = o->auto_reset;
    s->using_moving_camera = o->moving_cam;
    s->median_blur_kernel_size = o->median_k;
    s->n_local_words = (int32_t)o->L;
    s->n_global_words = (int32_t)o->G;
    s->last_nonflat_ratio = o->last_nonflat_ratio;
    s->n_relevant_px = o->n_rel;
    s->orig_roi_px = o->orig_roi;
    s->ds_roi_px = o->ds_roi_count;
    s->stat_words_scanned = o->st_words_scanned;
    s->stat_gdict_events = o->st_gdict_events;
    s->stat_nb_updates = o->st_nb_updates;
}
