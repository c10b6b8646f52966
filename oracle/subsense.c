/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * Plain-C restatement of BackgroundSubtractorSuBSENSE (plstcharles/litiv,
 * modules/video/src/BackgroundSubtractorSuBSENSE.cpp) together with its base
 * classes (BackgroundSubtractionUtils.cpp, BackgroundSubtractorLBSP.cpp), the
 * LBSP helpers (modules/features2d/include/litiv/features2d/LBSP.hpp), the
 * sampling helpers (modules/utils/include/litiv/utils/opencv.hpp:859-966) and
 * the OpenCV image operations the path calls. It keeps the reference's
 * sequential raster scan, its state layout (one full-frame map per quantity,
 * N sample images) and its floating-point operation order; it must be built
 * with -ffp-contract=off so that no multiply-add is fused.
 *
 * rand() is replaced by the counter-based generator of philox.h.
 *
 * OpenCV is not available, so the OpenCV calls are written here from their
 * documented definitions (each stated beside the function); their parity with
 * the real OpenCV is unpinned.
 */
#include "oracle.h"
#include "philox.h"
#include "common.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

/* constants of BackgroundSubtractorSuBSENSE.cpp:26-55 */
#define GHOSTDET_D_MAX (0.010f)
#define GHOSTDET_S_MIN (0.995f)
#define FEEDBACK_R_VAR (0.01f)
#define FEEDBACK_V_INCR (1.000f)
#define FEEDBACK_V_DECR (0.100f)
#define FEEDBACK_T_DECR (0.2500f)
#define FEEDBACK_T_INCR (0.5000f)
#define FEEDBACK_T_LOWER (2.0000f)
#define FEEDBACK_T_UPPER (256.00f)
#define UNSTABLE_REG_RATIO_MIN (0.100f)
#define UNSTABLE_REG_RDIST_MIN (3.000f)
#define LBSPDESC_NONZERO_RATIO_MIN (0.100f)
#define LBSPDESC_NONZERO_RATIO_MAX (0.500f)
#define DEFAULT_FRAME_AREA (320 * 240)
#define DS_RATIO 8



struct osub {
    osub_params p;
    int initialized;
    int W, H, C;
    size_t npx;
    uint8_t* roi;
    size_t* pxlut;
    size_t n_rel, orig_roi;
    uint8_t lut[256];
    size_t frame_idx, frames_since_reset, cooldown;
    int auto_reset, lr_scaling, use3x3, median_k;
    float t_lo, t_hi, last_nz_ratio;
    int ds_w, ds_h;
    float *R, *V, *T, *Dlast, *DminLT, *DminST, *RawLT, *RawST, *FinLT, *FinST;
    float *dsLT, *dsST;
    uint8_t* dsframe;
    uint8_t *unstable, *blinks, *lastRawFG, *lastFG, *lastFGdilInv, *lastRawBlink;
    uint8_t *currBlink, *preflood, *holes, *dil, *tmp8, *visited;
    int* bfs;
    uint8_t* lastColor;
    uint16_t* lastDesc;
    uint8_t* scol;
    uint16_t* sdesc;
    uint32_t* kctr;
    uint32_t ksent;
    uint32_t cache_px, cache_blk, cache_out[4];
    int cache_valid;
    uint64_t last_nz, last_colordiff, st_samples, st_writes;
};

void ophilox_block(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) { ophilox4x32_10(ctr, key, out); }

/* one rand() call of the reference, attributed to pixel px (or the frame-level sentinel) */
static int odraw(osub_t* o, size_t px) {
    uint32_t p32, *kp;
    if (px == (size_t)-1) {
        p32 = OPHILOX_SENTINEL_PX;
        kp = &o->ksent;
    } else {
        p32 = (uint32_t)px;
        kp = &o->kctr[px];
    }
    const uint32_t k = (*kp)++;
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

static void reset_draw_counters(osub_t* o) {
    memset(o->kctr, 0, o->npx * sizeof(uint32_t));
    o->ksent = 0;
    o->cache_valid = 0;
}


void osample_pos_7x7(int rnd, int x0, int y0, int W, int H, int* sx, int* sy) {
    sample_pos_7x7(rnd, sx, sy, x0, y0, LBSP_BORDER, W, H);
}
void oneighbor_pos(int rnd, int use3x3, int x0, int y0, int W, int H, int* nx, int* ny) {
    neighbor_pos(rnd, use3x3, nx, ny, x0, y0, LBSP_BORDER, W, H);
}


void olbsp_compute2(const uint8_t* img, int W, int H, int C, long abs_thr, float rel_thr, size_t offset,
                    uint16_t* desc) {
    /* lbsp_computeImpl, LBSP.cpp:102-152 */
    uint8_t vals[16];
    const uint8_t t = (uint8_t)(abs_thr < 0 ? 0 : abs_thr > 255 ? 255 : abs_thr);
    for (int y = LBSP_BORDER; y < H - LBSP_BORDER; ++y)
        for (int x = LBSP_BORDER; x < W - LBSP_BORDER; ++x)
            for (int c = 0; c < C; ++c) {
                const uint8_t ref = img[((size_t)y * W + x) * C + c];
                const uint8_t thr = abs_thr >= 0 ? t : sat_u8f((float)ref * rel_thr + (float)offset);
                lbsp_lookup(img, W, C, x, y, c, vals);
                desc[((size_t)y * W + x) * C + c] = lbsp_threshold(vals, ref, thr);
            }
}

void osub_default_params(osub_params* p) {
    p->desc_dist_threshold_offset = 3;
    p->min_color_dist_threshold = 30;
    p->bg_samples = 50;
    p->required_bg_samples = 2;
    p->samples_for_moving_avgs = 100;
    p->rel_lbsp_threshold = 0.333f;
    p->lbsp_threshold_offset = 0;
    p->default_median_blur_kernel_size = 9;
    p->seed = 0;
}

static void free_state(osub_t* o) {
    void* ptrs[] = {o->roi, o->pxlut, o->R, o->V, o->T, o->Dlast, o->DminLT, o->DminST, o->RawLT, o->RawST,
                    o->FinLT, o->FinST, o->dsLT, o->dsST, o->dsframe, o->unstable, o->blinks, o->lastRawFG,
                    o->lastFG, o->lastFGdilInv, o->lastRawBlink, o->currBlink, o->preflood, o->holes, o->dil,
                    o->tmp8, o->visited, o->bfs, o->lastColor, o->lastDesc, o->scol, o->sdesc, o->kctr};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    osub_params p = o->p;
    memset(o, 0, sizeof(*o));
    o->p = p;
}

osub_t* osub_create(const osub_params* p) {
    /* constructor checks, BackgroundSubtractorSuBSENSE.cpp:76-77 and BackgroundSubtractorLBSP.hpp:53 */
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return NULL;
    if (p->min_color_dist_threshold == 0 && p->desc_dist_threshold_offset == 0) return NULL;
    if (!(p->rel_lbsp_threshold >= 0)) return NULL;
    osub_t* o = (osub_t*)calloc(1, sizeof(osub_t));
    o->p = *p;
    return o;
}

void osub_destroy(osub_t* o) {
    if (!o) return;
    free_state(o);
    free(o);
}

void osub_set_automatic_model_reset(osub_t* o, int enabled) { o->auto_reset = enabled ? 1 : 0; }

/* ---- OpenCV operations used by the path (definitions stated; parity vs OpenCV unpinned) ---- */



/* cv::floodFill(img, Point(0,0), 255) (4-connectivity, zero tolerances) followed by
 * cv::bitwise_not: the result is 255 exactly at the pixels that hold 0 and are not
 * 4-connected through 0-pixels to (0,0). */
static void flood_holes(osub_t* o, const uint8_t* pre, uint8_t* holes) {
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




/* ---- initialize ---- */

int osub_initialize(osub_t* o, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    /* IIBackgroundSubtractor::initialize_common, BackgroundSubtractionUtils.cpp:70-155 */
    if (!img || W <= 0 || H <= 0) return OSUB_EBADARG;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED; /* 8UC4 is accepted by the base but apply() has no 4ch loop */
    const size_t npx = (size_t)W * H;
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
        /* dilate by m_nROIBorderSize (=2) iterations, /2, OR (BackgroundSubtractionUtils.cpp:94-95):
         * `Mat / 2` is OpenCV's scaling expression, saturate_cast(v * 0.5) rounded half to even, so the
         * pixels near the ROI edge get 128 (255 / 2 = 127.5) */
        uint8_t* d = (uint8_t*)malloc(npx);
        uint8_t* t = (uint8_t*)malloc(npx);
        box_minmax(roi, d, t, W, H, LBSP_BORDER, 1);
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
    /* validateROI, BackgroundSubtractionUtils.cpp:28-36: keep only [2, W-2) x [2, H-2) */
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
    free_state(o);
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
    o->pxlut = (size_t*)malloc(fin * sizeof(size_t));
    for (size_t i = 0, m = 0; i < npx; ++i)
        if (newroi[i]) o->pxlut[m++] = i;
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
    /* BackgroundSubtractorSuBSENSE::initialize, BackgroundSubtractorSuBSENSE.cpp:110-182 */
    o->last_nz_ratio = 0.0f;
    const int area = W * H;
    if (orig >= npx / 2 && (int)npx >= DEFAULT_FRAME_AREA) {
        o->lr_scaling = 1;
        o->auto_reset = 1;
        o->use3x3 = !(area > DEFAULT_FRAME_AREA * 2);
        int raw = (int)floorf((float)area / DEFAULT_FRAME_AREA + 0.5f) + o->p.default_median_blur_kernel_size;
        raw = raw < 14 ? raw : 14;
        o->median_k = (raw % 2) ? raw : raw - 1;
        o->t_lo = FEEDBACK_T_LOWER;
        o->t_hi = FEEDBACK_T_UPPER;
    } else {
        o->lr_scaling = 0;
        o->auto_reset = 0;
        o->use3x3 = 1;
        o->median_k = o->p.default_median_blur_kernel_size;
        o->t_lo = FEEDBACK_T_LOWER * 2;
        o->t_hi = FEEDBACK_T_UPPER * 2;
    }
    float** fmaps[] = {&o->R, &o->V, &o->T, &o->Dlast, &o->DminLT, &o->DminST, &o->RawLT, &o->RawST, &o->FinLT, &o->FinST};
    for (size_t m = 0; m < sizeof(fmaps) / sizeof(fmaps[0]); ++m) *fmaps[m] = (float*)calloc(npx, sizeof(float));
    for (size_t i = 0; i < npx; ++i) {
        o->T[i] = o->t_lo;
        o->R[i] = 1.0f;
        o->V[i] = 10.0f;
    }
    o->ds_w = W / DS_RATIO;
    o->ds_h = H / DS_RATIO;
    const size_t nds = (size_t)o->ds_w * o->ds_h * C;
    o->dsLT = (float*)calloc(nds ? nds : 1, sizeof(float));
    o->dsST = (float*)calloc(nds ? nds : 1, sizeof(float));
    o->dsframe = (uint8_t*)calloc(nds ? nds : 1, 1);
    uint8_t** bmaps[] = {&o->unstable, &o->blinks,   &o->lastRawFG, &o->lastFG, &o->lastFGdilInv, &o->lastRawBlink,
                         &o->currBlink, &o->preflood, &o->holes,     &o->dil,    &o->tmp8,         &o->visited};
    for (size_t m = 0; m < sizeof(bmaps) / sizeof(bmaps[0]); ++m) *bmaps[m] = (uint8_t*)calloc(npx, 1);
    o->bfs = (int*)malloc(npx * sizeof(int));
    o->scol = (uint8_t*)calloc(o->p.bg_samples * npx * C, 1);
    o->sdesc = (uint16_t*)calloc(o->p.bg_samples * npx * C, sizeof(uint16_t));
    o->kctr = (uint32_t*)calloc(npx, sizeof(uint32_t));
    o->initialized = 1;
    reset_draw_counters(o);
    osub_refresh_model(o, 1.0f, 0);
    return OSUB_OK;
}

/* BackgroundSubtractorSuBSENSE::refreshModel, BackgroundSubtractorSuBSENSE.cpp:80-105 */
int osub_refresh_model(osub_t* o, float frac, int force) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!(frac > 0.0f && frac <= 1.0f)) return OSUB_EBADARG;
    const size_t N = o->p.bg_samples, C = (size_t)o->C;
    const size_t nref = frac < 1.0f ? (size_t)(frac * (float)N) : N;
    const size_t start = frac < 1.0f ? (size_t)odraw(o, (size_t)-1) % N : 0;
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        if (force || !o->lastFG[px]) {
            const int x0 = (int)(px % o->W), y0 = (int)(px / o->W);
            for (size_t s = start; s < start + nref; ++s) {
                int sx, sy;
                sample_pos_7x7(odraw(o, px), &sx, &sy, x0, y0, LBSP_BORDER, o->W, o->H);
                const size_t spx = (size_t)o->W * sy + sx;
                if (force || !o->lastFG[spx]) {
                    const size_t rs = s % N;
                    for (size_t c = 0; c < C; ++c) {
                        o->scol[rs * o->npx * C + px * C + c] = o->lastColor[spx * C + c];
                        o->sdesc[rs * o->npx * C + px * C + c] = o->lastDesc[spx * C + c];
                    }
                }
            }
        }
    }
    return OSUB_OK;
}

static void write_sample(osub_t* o, size_t s, size_t px, const uint8_t* col, const uint16_t* desc) {
    const size_t C = (size_t)o->C;
    for (size_t c = 0; c < C; ++c) {
        o->sdesc[s * o->npx * C + px * C + c] = desc[c];
        o->scol[s * o->npx * C + px * C + c] = col[c];
    }
    o->st_writes++;
}

/* ---- apply ---- */

int osub_apply(osub_t* o, const uint8_t* img, uint8_t* mask, double lr) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!img || !mask) return OSUB_EBADARG;
    const int W = o->W, H = o->H;
    const size_t C = (size_t)o->C, N = o->p.bg_samples, npx = o->npx, nreq = o->p.required_bg_samples;
    const size_t colMax1 = 255, descMax1 = 16, colMax3 = colMax1 * 3, descMax3 = descMax1 * 3;
    const size_t minColor = o->p.min_color_dist_threshold, descOff = o->p.desc_dist_threshold_offset;
    const size_t stabColorOff = minColor / 5; /* STAB_COLOR_DIST_OFFSET */
    memset(mask, 0, npx);
    size_t nz = 0;
    ++o->frame_idx;
    reset_draw_counters(o);
    const size_t nmv = o->p.samples_for_moving_avgs;
    const float fLT = 1.0f / (float)(o->frame_idx < nmv ? o->frame_idx : nmv);
    const float fST = 1.0f / (float)(o->frame_idx < nmv / 4 ? o->frame_idx : nmv / 4);
    uint8_t vals[3][16];
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const int x = (int)(px % W), y = (int)(px / W);
        const uint8_t* curr = img + px * C;
        float* R = &o->R[px];
        float* V = &o->V[px];
        float* T = &o->T[px];
        float* Dl = &o->Dlast[px];
        float* DLT = &o->DminLT[px];
        float* DST = &o->DminST[px];
        float* RLT = &o->RawLT[px];
        float* RST = &o->RawST[px];
        const float FLT = o->FinLT[px], FST = o->FinST[px];
        uint8_t* lastCol = o->lastColor + px * C;
        uint16_t* lastDesc = o->lastDesc + px * C;
        /* thresholds, :222-223 (1ch) and :355-359 (3ch), from the unstable flag of the previous frame */
        const size_t colThr =
            (size_t)((*R * (float)minColor) - (float)((size_t)(!o->unstable[px]) * stabColorOff));
        const size_t descThr = ((size_t)1 << (size_t)floorf(*R + 0.5f)) + descOff + (size_t)o->unstable[px] * descOff;
        uint16_t intra[3];
        for (size_t c = 0; c < C; ++c) {
            lbsp_lookup(img, W, (int)C, x, y, (int)c, vals[c]);
            intra[c] = lbsp_threshold(vals[c], curr[c], o->lut[curr[c]]);
        }
        o->unstable[px] = (*R > UNSTABLE_REG_RDIST_MIN || (*RLT - FLT) > UNSTABLE_REG_RATIO_MIN ||
                           (*RST - FST) > UNSTABLE_REG_RATIO_MIN) ? 1 : 0;
        size_t nGood = 0, s = 0;
        size_t minDesc, minSum;
        float normLast;
        if (C == 1) {
            /* :228-253 */
            const size_t cthr = colThr / 2;
            minDesc = descMax1;
            minSum = colMax1;
            while (nGood < nreq && s < N) {
                const uint8_t bgc = o->scol[s * npx + px];
                const uint16_t bgd = o->sdesc[s * npx + px];
                const size_t colDist = absdiff(curr[0], bgc);
                if (colDist > cthr) goto fail1;
                {
                    const size_t intraD = popc16(intra[0] ^ bgd);
                    const uint16_t inter = lbsp_threshold(vals[0], bgc, o->lut[bgc]);
                    const size_t interD = popc16(inter ^ bgd);
                    const size_t descDist = (intraD + interD) / 2;
                    if (descDist > descThr) goto fail1;
                    size_t sumDist = (descDist / 4) * (colMax1 / descMax1) + colDist;
                    if (sumDist > colMax1) sumDist = colMax1;
                    if (sumDist > cthr) goto fail1;
                    if (minDesc > descDist) minDesc = descDist;
                    if (minSum > sumDist) minSum = sumDist;
                    nGood++;
                }
            fail1:
                s++;
            }
            normLast = ((float)absdiff(lastCol[0], curr[0]) / (float)colMax1 +
                        (float)popc16(lastDesc[0] ^ intra[0]) / (float)descMax1) / 2;
        } else {
            /* :366-395 */
            const size_t totColThr = colThr * 3, totDescThr = descThr * 3, scColThr = totColThr / 2;
            minDesc = descMax3;
            minSum = colMax3;
            while (nGood < nreq && s < N) {
                const uint16_t* bgd = o->sdesc + s * npx * 3 + px * 3;
                const uint8_t* bgc = o->scol + s * npx * 3 + px * 3;
                size_t totDesc = 0, totSum = 0;
                for (size_t c = 0; c < 3; ++c) {
                    const size_t colDist = absdiff(curr[c], bgc[c]);
                    if (colDist > scColThr) goto fail3;
                    const size_t intraD = popc16(intra[c] ^ bgd[c]);
                    const uint16_t inter = lbsp_threshold(vals[c], bgc[c], o->lut[bgc[c]]);
                    const size_t interD = popc16(inter ^ bgd[c]);
                    const size_t descDist = (intraD + interD) / 2;
                    size_t sumDist = (descDist / 2) * (colMax1 / descMax1) + colDist;
                    if (sumDist > colMax1) sumDist = colMax1;
                    if (sumDist > scColThr) goto fail3;
                    totDesc += descDist;
                    totSum += sumDist;
                }
                if (totDesc > totDescThr || totSum > totColThr) goto fail3;
                if (minDesc > totDesc) minDesc = totDesc;
                if (minSum > totSum) minSum = totSum;
                nGood++;
            fail3:
                s++;
            }
            /* lv::L1dist<3>(const uchar*, const uchar*) (math.hpp:226-232) accumulates in its Tout, which is
             * decltype(L1dist(uchar, uchar)) = unsigned char: the three-channel sum wraps modulo 256 */
            const size_t l1 = (uint8_t)(absdiff(lastCol[0], curr[0]) + absdiff(lastCol[1], curr[1]) + absdiff(lastCol[2], curr[2]));
            const size_t hd = popc16(lastDesc[0] ^ intra[0]) + popc16(lastDesc[1] ^ intra[1]) + popc16(lastDesc[2] ^ intra[2]);
            normLast = ((float)l1 / (float)colMax3 + (float)hd / (float)descMax3) / 2;
        }
        o->st_samples += s;
        const float colMax = (float)(C == 1 ? colMax1 : colMax3), descMax = (float)(C == 1 ? descMax1 : descMax3);
        *Dl = (*Dl) * (1.0f - fST) + normLast * fST;
        if (nGood < nreq) {
            /* foreground, :256-269 / :398-413 */
            const float md = ((float)minSum / colMax + (float)minDesc / descMax) / 2 + (float)(nreq - nGood) / (float)nreq;
            const float nmd = minf_std(1.0f, md);
            *DLT = (*DLT) * (1.0f - fLT) + nmd * fLT;
            *DST = (*DST) * (1.0f - fST) + nmd * fST;
            *RLT = (*RLT) * (1.0f - fLT) + fLT;
            *RST = (*RST) * (1.0f - fST) + fST;
            mask[px] = 255;
            if (o->cooldown && ((size_t)odraw(o, px) % (size_t)FEEDBACK_T_LOWER) == 0) {
                const size_t sr = (size_t)odraw(o, px) % N;
                write_sample(o, sr, px, curr, intra);
            }
        } else {
            /* background, :270-301 / :414-450 */
            const float nmd = ((float)minSum / colMax + (float)minDesc / descMax) / 2;
            *DLT = (*DLT) * (1.0f - fLT) + nmd * fLT;
            *DST = (*DST) * (1.0f - fST) + nmd * fST;
            *RLT = (*RLT) * (1.0f - fLT);
            *RST = (*RST) * (1.0f - fST);
            const size_t nLR = isinf(lr) ? SIZE_MAX : (lr > 0 ? (size_t)ceil(lr) : (size_t)ceilf(*T));
            if (((size_t)odraw(o, px) % nLR) == 0) {
                const size_t sr = (size_t)odraw(o, px) % N;
                write_sample(o, sr, px, curr, intra);
            }
            const int use3 = o->use3x3 && !o->unstable[px];
            int nx, ny;
            neighbor_pos(odraw(o, px), use3, &nx, &ny, x, y, LBSP_BORDER, W, H);
            const size_t nrand = (size_t)odraw(o, px);
            const size_t q = (size_t)W * ny + nx;
            const float qDlast = o->Dlast[q];
            const float qRawST = o->RawST[q];
            if ((nrand % (use3 ? nLR : (nLR / 2 + 1))) == 0 ||
                (qRawST > GHOSTDET_S_MIN && qDlast < GHOSTDET_D_MAX && (nrand % (size_t)o->t_lo) == 0)) {
                const size_t sr = (size_t)odraw(o, px) % N;
                write_sample(o, sr, q, curr, intra);
            }
        }
        /* feedback: T :302-311, v :312-318, R :319-325 */
        const float mn = minf_std(*DLT, *DST), mx = maxf_std(*DLT, *DST);
        if (o->lastFG[px] || (mn < UNSTABLE_REG_RATIO_MIN && mask[px])) {
            if (*T < o->t_hi) *T += FEEDBACK_T_INCR / (mx * (*V));
        } else if (*T > o->t_lo) {
            *T -= FEEDBACK_T_DECR * (*V) / mx;
        }
        if (*T < o->t_lo) *T = o->t_lo;
        else if (*T > o->t_hi) *T = o->t_hi;
        if (mx > UNSTABLE_REG_RATIO_MIN && o->blinks[px]) {
            *V += FEEDBACK_V_INCR;
        } else if (*V > FEEDBACK_V_DECR) {
            *V -= o->lastFG[px] ? FEEDBACK_V_DECR / 4 : o->unstable[px] ? FEEDBACK_V_DECR / 2 : FEEDBACK_V_DECR;
            if (*V < FEEDBACK_V_DECR) *V = FEEDBACK_V_DECR;
        }
        const double rx = (double)(1.0f + mn * 2);
        if ((double)*R < rx * rx) {
            *R += FEEDBACK_R_VAR * (*V - FEEDBACK_V_DECR);
        } else {
            *R -= FEEDBACK_R_VAR / (*V);
            if (*R < 1.0f) *R = 1.0f;
        }
        /* :326-329 / :475-480 */
        unsigned pc = 0;
        for (size_t c = 0; c < C; ++c) pc += popc16(intra[c]);
        if (pc >= (C == 1 ? 2u : 4u)) ++nz;
        for (size_t c = 0; c < C; ++c) {
            lastDesc[c] = intra[c];
            lastCol[c] = curr[c];
        }
    }
    /* post-processing, :536-554 */
    for (size_t i = 0; i < npx; ++i) {
        o->currBlink[i] = mask[i] ^ o->lastRawFG[i];
        o->blinks[i] = o->currBlink[i] | o->lastRawBlink[i];
        o->lastRawBlink[i] = o->currBlink[i];
        o->lastRawFG[i] = mask[i];
    }
    box_minmax(mask, o->dil, o->tmp8, W, H, 1, 1);          /* MORPH_CLOSE 3x3: dilate ... */
    box_minmax(o->dil, o->preflood, o->tmp8, W, H, 1, 0);   /* ... then erode */
    flood_holes(o, o->preflood, o->holes);
    box_minmax(o->preflood, o->dil, o->tmp8, W, H, 3, 0);   /* erode x3 of the closed mask */
    for (size_t i = 0; i < npx; ++i) mask[i] = mask[i] | o->holes[i] | o->dil[i];
    median_binary(mask, o->lastFG, (uint16_t*)o->bfs, W, H, o->median_k);
    box_minmax(o->lastFG, o->dil, o->tmp8, W, H, 3, 1);     /* dilate x3 */
    for (size_t i = 0; i < npx; ++i) {
        o->blinks[i] &= o->lastFGdilInv[i];                  /* previous frame's inverted dilated mask */
        o->lastFGdilInv[i] = (uint8_t)~o->dil[i];
        o->blinks[i] &= o->lastFGdilInv[i];
        mask[i] = o->lastFG[i];
    }
    add_weighted_mask(o->FinLT, o->lastFG, npx, (double)(1.0f - fLT), (1.0 / 255) * (double)fLT);
    add_weighted_mask(o->FinST, o->lastFG, npx, (double)(1.0f - fST), (1.0 / 255) * (double)fST);
    /* LBSP threshold LUT adaptation, :555-566 */
    const float nzRatio = (float)nz / (float)o->n_rel;
    const float rel = o->p.rel_lbsp_threshold;
    if (nzRatio < LBSPDESC_NONZERO_RATIO_MIN && o->last_nz_ratio < LBSPDESC_NONZERO_RATIO_MIN) {
        for (int t = 0; t <= 255; ++t)
            if (o->lut[t] > sat_u8d((double)o->p.lbsp_threshold_offset + ceil((double)((float)t * rel / 4))))
                --o->lut[t];
    } else if (nzRatio > LBSPDESC_NONZERO_RATIO_MAX && o->last_nz_ratio > LBSPDESC_NONZERO_RATIO_MAX) {
        for (int t = 0; t <= 255; ++t)
            if (o->lut[t] < sat_u8f((float)o->p.lbsp_threshold_offset + 255 * rel)) ++o->lut[t];
    }
    o->last_nz_ratio = nzRatio;
    o->last_nz = nz;
    o->last_colordiff = 0;
    /* frame-level analysis, :567-611 */
    if (o->lr_scaling) {
        if (!resize_area_div8(img, W, H, (int)C, o->dsframe, o->ds_w, o->ds_h)) return OSUB_EBADARG;
        const size_t nds = (size_t)o->ds_w * o->ds_h * C;
        accumulate_weighted(o->dsframe, o->dsLT, nds, (double)fLT);
        accumulate_weighted(o->dsframe, o->dsST, nds, (double)fST);
        size_t tot = 0;
        for (size_t i = 0; i < (size_t)o->ds_w * o->ds_h; ++i) {
            if (C == 1) {
                tot += (size_t)fabsf(o->dsST[i] - o->dsLT[i]) / 2;
            } else {
                const size_t d0 = (size_t)fabsf(o->dsST[i * 3 + 0] - o->dsLT[i * 3 + 0]);
                const size_t d1 = (size_t)fabsf(o->dsST[i * 3 + 1] - o->dsLT[i * 3 + 1]);
                const size_t d2 = (size_t)fabsf(o->dsST[i * 3 + 2] - o->dsLT[i * 3 + 2]);
                const size_t m12 = d1 > d2 ? d1 : d2;
                tot += d0 > m12 ? d0 : m12;
            }
        }
        o->last_colordiff = tot;
        const float ratio = (float)tot / (float)(o->ds_w * o->ds_h);
        const size_t thr = minColor / 2; /* FRAMELEVEL_MIN_COLOR_DIFF_THRESHOLD */
        if (o->auto_reset) {
            if (o->frames_since_reset > 1000) {
                o->auto_reset = 0;
            } else if (ratio >= (float)thr && o->cooldown == 0) {
                o->frames_since_reset = 0;
                osub_refresh_model(o, 0.1f, 0);
                o->cooldown = nmv / 4;
                for (size_t i = 0; i < npx; ++i) o->T[i] = 1.0f;
            } else {
                ++o->frames_since_reset;
            }
        } else if (ratio >= (float)(thr * 2)) {
            o->frames_since_reset = 0;
            o->auto_reset = 1;
        }
        if (ratio >= (float)(thr / 2)) {
            /* the shift count is taken modulo 32, as the x86-64 and AArch64 shift instructions do */
            const int sh = ((int)(ratio / 2)) & 31;
            const int lo = (int)FEEDBACK_T_LOWER >> sh, hi = (int)FEEDBACK_T_UPPER >> sh;
            o->t_lo = (float)(lo > 1 ? lo : 1);
            o->t_hi = (float)(hi > 1 ? hi : 1);
        } else {
            o->t_lo = FEEDBACK_T_LOWER;
            o->t_hi = FEEDBACK_T_UPPER;
        }
        if (o->cooldown > 0) --o->cooldown;
    }
    return OSUB_OK;
}

/* getBackgroundImage, :614-630: per-pixel mean of the N colour samples, accumulated in float
 * in sample order (+= v/N), then convertTo(CV_8U) (cvRound, saturate) */
/* setROI, BackgroundSubtractionUtils.cpp:38-48, with validateROI :28-36 */
int osub_set_roi(osub_t* o, const uint8_t* roi, int W, int H) {
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
        osub_get_background(o, bg);
        const int st = osub_initialize(o, bg, W, H, o->C, r);
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

int osub_get_background(const osub_t* o, uint8_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t n = o->npx * o->C, N = o->p.bg_samples;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->scol[s * n + i]) / (float)N;
        out[i] = sat_u8f(acc);
    }
    return OSUB_OK;
}

/* getBackgroundDescriptorsImage, :632-649 (same, with a CV_16U conversion) */
int osub_get_background_descriptors(const osub_t* o, uint16_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t n = o->npx * o->C, N = o->p.bg_samples;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->sdesc[s * n + i]) / (float)N;
        out[i] = sat_u16f(acc);
    }
    return OSUB_OK;
}

const void* osub_map(const osub_t* o, int which, size_t* nbytes) {
    const size_t npx = o->npx, C = (size_t)o->C, N = o->p.bg_samples;
    const size_t nds = (size_t)o->ds_w * o->ds_h * C;
    const void* p = NULL;
    size_t n = 0;
    switch (which) {
        case OSUB_MAP_R: p = o->R; n = npx * 4; break;
        case OSUB_MAP_V: p = o->V; n = npx * 4; break;
        case OSUB_MAP_T: p = o->T; n = npx * 4; break;
        case OSUB_MAP_DLAST: p = o->Dlast; n = npx * 4; break;
        case OSUB_MAP_DMIN_LT: p = o->DminLT; n = npx * 4; break;
        case OSUB_MAP_DMIN_ST: p = o->DminST; n = npx * 4; break;
        case OSUB_MAP_RAW_LT: p = o->RawLT; n = npx * 4; break;
        case OSUB_MAP_RAW_ST: p = o->RawST; n = npx * 4; break;
        case OSUB_MAP_FIN_LT: p = o->FinLT; n = npx * 4; break;
        case OSUB_MAP_FIN_ST: p = o->FinST; n = npx * 4; break;
        case OSUB_MAP_UNSTABLE: p = o->unstable; n = npx; break;
        case OSUB_MAP_BLINKS: p = o->blinks; n = npx; break;
        case OSUB_MAP_LAST_RAW_FG: p = o->lastRawFG; n = npx; break;
        case OSUB_MAP_LAST_FG: p = o->lastFG; n = npx; break;
        case OSUB_MAP_LAST_FG_DIL_INV: p = o->lastFGdilInv; n = npx; break;
        case OSUB_MAP_LAST_RAW_BLINK: p = o->lastRawBlink; n = npx; break;
        case OSUB_MAP_ROI: p = o->roi; n = npx; break;
        case OSUB_MAP_LAST_COLOR: p = o->lastColor; n = npx * C; break;
        case OSUB_MAP_LAST_DESC: p = o->lastDesc; n = npx * C * 2; break;
        case OSUB_MAP_SAMPLE_COLOR: p = o->scol; n = N * npx * C; break;
        case OSUB_MAP_SAMPLE_DESC: p = o->sdesc; n = N * npx * C * 2; break;
        case OSUB_MAP_DS_LT: p = o->dsLT; n = nds * 4; break;
        case OSUB_MAP_DS_ST: p = o->dsST; n = nds * 4; break;
        case OSUB_MAP_LUT: p = o->lut; n = 256; break;
        default: break;
    }
    if (nbytes) *nbytes = p ? n : 0;
    return p;
}

void osub_get_scalars(const osub_t* o, osub_scalars* s) {
    memset(s, 0, sizeof(*s));
    s->frame_idx = o->frame_idx;
    s->frames_since_last_reset = o->frames_since_reset;
    s->model_reset_cooldown = o->cooldown;
    s->auto_model_reset_enabled = o->auto_reset;
    s->learning_rate_scaling_enabled = o->lr_scaling;
    s->use_3x3_spread = o->use3x3;
    s->median_blur_kernel_size = o->median_k;
    s->lr_lower_cap = o->t_lo;
    s->lr_upper_cap = o->t_hi;
    s->last_nonzero_desc_ratio = o->last_nz_ratio;
    s->nonzero_desc_count = o->last_nz;
    s->tot_color_diff = o->last_colordiff;
    s->n_relevant_px = o->n_rel;
    s->orig_roi_px = o->orig_roi;
    s->stat_samples_evaluated = o->st_samples;
    s->stat_sample_writes = o->st_writes;
}
