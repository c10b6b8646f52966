/* ORACLE (test infrastructure only; never linked into the product library).
 *
 * CPU restatement of the reference's LOBSTER background subtraction, the non-parallel path of
 * BackgroundSubtractorLOBSTER (modules/video/src/BackgroundSubtractorLOBSTER.cpp:410-620), on top
 * of the same LBSP / sampling / ROI definitions as the SuBSENSE restatement (common.h, and
 * BackgroundSubtractionUtils.cpp:70-155 / BackgroundSubtractorLBSP.cpp:21-65 for initialize_common).
 *
 * rand() is draw k of pixel p in frame t of the counter-based generator (philox.h). LOBSTER keeps no
 * frame counter of its own (apply() never advances m_nFrameIdx), so t counts apply() calls here:
 * initialize() and refreshModel() before the first apply() are frame 0, the i-th apply() frame i,
 * and a refreshModel() between frames continues the draw counters of the last frame.
 * Pinned to the reference by tests/test_oracle_reference.py (oracle/_ref, rlob_*).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "common.h"
#include "oracle.h"
#include "philox.h"

struct olob {
    olob_params p;
    int initialized;
    int W, H, C;
    size_t npx, n_rel, orig_roi;
    uint8_t* roi;
    size_t* pxlut;
    uint8_t lut[256];
    uint8_t *lastColor, *lastFG, *rawFG;
    uint16_t* lastDesc;
    uint16_t* colcnt;
    uint8_t* scol;   /* [N][npx*C] */
    uint16_t* sdesc; /* [N][npx*C] */
    uint32_t* kctr;
    uint32_t ksent;
    uint64_t frames; /* apply() calls since initialize(): the generator's frame */
    int cache_valid;
    uint32_t cache_px, cache_blk, cache_out[4];
    uint64_t st_samples, st_writes;
};

/* one rand() call of the reference, attributed to pixel px (or the frame-level sentinel) */
static int ldraw(olob_t* o, size_t px) {
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
        const uint32_t ctr[4] = {blk, p32, (uint32_t)o->frames, 0u};
        const uint32_t key[2] = {(uint32_t)o->p.seed, (uint32_t)(o->p.seed >> 32)};
        ophilox4x32_10(ctr, key, o->cache_out);
        o->cache_px = p32;
        o->cache_blk = blk;
        o->cache_valid = 1;
    }
    return (int)(o->cache_out[k & 3u] & 0x7fffffffu);
}

static void start_frame(olob_t* o) {
    memset(o->kctr, 0, o->npx * sizeof(uint32_t));
    o->ksent = 0;
    o->cache_valid = 0;
}

void olob_default_params(olob_params* p) {
    /* BackgroundSubtractorLOBSTER.hpp:22-31 and BackgroundSubtractorLBSP.hpp:23-28 */
    p->desc_dist_threshold = 4;
    p->color_dist_threshold = 30;
    p->bg_samples = 35;
    p->required_bg_samples = 2;
    p->rel_lbsp_threshold = 0.333f;
    p->lbsp_threshold_offset = 0;
    p->default_median_blur_kernel_size = 9;
    p->seed = 0;
}

static void lob_free(olob_t* o) {
    void* ptrs[] = {o->roi, o->pxlut, o->lastColor, o->lastFG, o->rawFG, o->lastDesc, o->colcnt, o->scol, o->sdesc, o->kctr};
    for (size_t i = 0; i < sizeof(ptrs) / sizeof(ptrs[0]); ++i) free(ptrs[i]);
    olob_params p = o->p;
    memset(o, 0, sizeof(*o));
    o->p = p;
}

olob_t* olob_create(const olob_params* p) {
    /* constructor checks, BackgroundSubtractorLOBSTER.cpp:21-30 and BackgroundSubtractorLBSP.hpp:53 */
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return NULL;
    if (p->color_dist_threshold == 0 && p->desc_dist_threshold == 0) return NULL;
    if (!(p->rel_lbsp_threshold >= 0)) return NULL;
    olob_t* o = (olob_t*)calloc(1, sizeof(olob_t));
    o->p = *p;
    return o;
}

void olob_destroy(olob_t* o) {
    if (!o) return;
    lob_free(o);
    free(o);
}

/* LBSP descriptor of channel c at (x, y) of an image, threshold from the LUT of its own value
 * (LBSP::computeDescriptor<C>, LBSP.hpp:159-191, as called at BackgroundSubtractorLOBSTER.cpp:427-432) */
static uint16_t lob_desc_at(const olob_t* o, const uint8_t* img, int x, int y, int c) {
    uint8_t vals[16];
    lbsp_lookup(img, o->W, o->C, x, y, c, vals);
    const uint8_t ref = img[((size_t)y * o->W + x) * o->C + c];
    return lbsp_threshold(vals, ref, o->lut[ref]);
}

/* BackgroundSubtractorLOBSTER::refreshModel, BackgroundSubtractorLOBSTER.cpp:410-440 */
int olob_refresh_model(olob_t* o, float frac, int force) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!(frac > 0.0f && frac <= 1.0f)) return OSUB_EBADARG;
    const size_t N = o->p.bg_samples, C = (size_t)o->C, npx = o->npx;
    const size_t nref = frac < 1.0f ? (size_t)(frac * (float)N) : N;
    const size_t start = frac < 1.0f ? (size_t)ldraw(o, (size_t)-1) % N : 0;
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        if (!(force || !o->lastFG[px])) continue;
        const int x0 = (int)(px % o->W), y0 = (int)(px / o->W);
        for (size_t s = start; s < start + nref; ++s) {
            int sx, sy;
            sample_pos_7x7(ldraw(o, px), &sx, &sy, x0, y0, LBSP_BORDER, o->W, o->H);
            const size_t spx = (size_t)o->W * sy + sx;
            if (!(force || !o->lastFG[spx])) continue;
            const size_t rs = s % N;
            for (size_t c = 0; c < C; ++c) {
                o->scol[rs * npx * C + px * C + c] = o->lastColor[spx * C + c];
                /* the descriptor of the last colour frame at the sample position, kept in the last
                 * descriptor frame (:427-432) and copied into the sample (:433) */
                o->lastDesc[spx * C + c] = lob_desc_at(o, o->lastColor, sx, sy, (int)c);
                o->sdesc[rs * npx * C + px * C + c] = o->lastDesc[spx * C + c];
            }
        }
    }
    return OSUB_OK;
}

/* BackgroundSubtractorLOBSTER::initialize, BackgroundSubtractorLOBSTER.cpp:442-457 */
int olob_initialize(olob_t* o, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    /* IIBackgroundSubtractor::initialize_common, BackgroundSubtractionUtils.cpp:70-155 */
    if (!img || W <= 0 || H <= 0) return OSUB_EBADARG;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED; /* apply() has 1- and 3-channel loops only */
    const size_t npx = (size_t)W * H;
    uint8_t* newroi = (uint8_t*)malloc(npx);
    if (!roi && o->roi && o->W == W && o->H == H) {
        memcpy(newroi, o->roi, npx); /* the last validated ROI is reused (:86-87) */
    } else if (!roi) {
        memset(newroi, 255, npx);
    } else {
        for (size_t i = 0; i < npx; ++i)
            if (roi[i] != 0 && roi[i] != 255) {
                free(newroi);
                return OSUB_EBADARG;
            }
        /* dilate by m_nROIBorderSize (=2) iterations, Mat/2 (round half to even: 128), OR (:94-95) */
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
    /* validateROI, BackgroundSubtractionUtils.cpp:28-36 */
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
    lob_free(o);
    o->W = W;
    o->H = H;
    o->C = C;
    o->npx = npx;
    o->roi = newroi;
    o->orig_roi = orig;
    o->n_rel = fin;
    o->frames = 0;
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
    o->lastFG = (uint8_t*)calloc(npx, 1);
    o->rawFG = (uint8_t*)calloc(npx, 1);
    o->colcnt = (uint16_t*)calloc(npx, sizeof(uint16_t));
    /* :446-453: all samples zero, then the model is refreshed from the frame (:455) */
    o->scol = (uint8_t*)calloc(o->p.bg_samples * npx * C, 1);
    o->sdesc = (uint16_t*)calloc(o->p.bg_samples * npx * C, sizeof(uint16_t));
    o->kctr = (uint32_t*)calloc(npx, sizeof(uint32_t));
    o->initialized = 1;
    start_frame(o);
    return olob_refresh_model(o, 1.0f, 1);
}

/* BackgroundSubtractorLOBSTER::apply, BackgroundSubtractorLOBSTER.cpp:459-581 */
int olob_apply(olob_t* o, const uint8_t* img, uint8_t* mask, double lr) {
    if (!o->initialized) return OSUB_ENOTINIT;
    if (!img || !mask || !(lr > 0)) return OSUB_EBADARG; /* :462-463 */
    const int W = o->W, H = o->H;
    const size_t C = (size_t)o->C, N = o->p.bg_samples, npx = o->npx, nreq = o->p.required_bg_samples;
    const size_t nLR = isinf(lr) ? (size_t)-1 : (size_t)ceil(lr); /* :470 */
    ++o->frames;
    start_frame(o);
    memset(o->rawFG, 0, npx);
    uint8_t vals[3][16];
    uint16_t intra[3];
    for (size_t m = 0; m < o->n_rel; ++m) {
        const size_t px = o->pxlut[m];
        const int x = (int)(px % W), y = (int)(px / W);
        const uint8_t* curr = img + px * C;
        for (size_t c = 0; c < C; ++c) lbsp_lookup(img, W, (int)C, x, y, (int)c, vals[c]);
        size_t nGood = 0, s = 0;
        if (C == 1) {
            /* :474-496 */
            const size_t colThr = o->p.color_dist_threshold / 2, descThr = o->p.desc_dist_threshold;
            while (nGood < nreq && s < N) {
                const uint8_t bgc = o->scol[s * npx + px];
                const uint16_t bgd = o->sdesc[s * npx + px];
                ++o->st_samples;
                if (absdiff(curr[0], bgc) <= colThr &&
                    (size_t)popc16(lbsp_threshold(vals[0], bgc, o->lut[bgc]) ^ bgd) <= descThr)
                    ++nGood;
                ++s;
            }
        } else {
            /* :517-541 */
            const size_t descThr = o->p.desc_dist_threshold * 3, colThr = o->p.color_dist_threshold * 3;
            const size_t scDescThr = descThr / 2, scColThr = colThr / 2;
            while (nGood < nreq && s < N) {
                const uint8_t* bgc = o->scol + s * npx * 3 + px * 3;
                const uint16_t* bgd = o->sdesc + s * npx * 3 + px * 3;
                size_t totCol = 0, totDesc = 0;
                int ok = 1;
                ++o->st_samples;
                for (size_t c = 0; c < 3 && ok; ++c) {
                    const size_t colDist = absdiff(curr[c], bgc[c]);
                    if (colDist > scColThr) {
                        ok = 0;
                        break;
                    }
                    const size_t descDist = popc16(lbsp_threshold(vals[c], bgc[c], o->lut[bgc[c]]) ^ bgd[c]);
                    if (descDist > scDescThr) {
                        ok = 0;
                        break;
                    }
                    totCol += colDist;
                    totDesc += descDist;
                }
                if (ok && totDesc <= descThr && totCol <= colThr) ++nGood;
                ++s;
            }
        }
        if (nGood < nreq) {
            o->rawFG[px] = 255;
            continue;
        }
        /* model updates with the current pixel (:497-513 / :545-575) */
        for (size_t c = 0; c < C; ++c) intra[c] = lbsp_threshold(vals[c], curr[c], o->lut[curr[c]]);
        if (((size_t)ldraw(o, px) % nLR) == 0) {
            const size_t rs = (size_t)ldraw(o, px) % N;
            for (size_t c = 0; c < C; ++c) {
                o->scol[rs * npx * C + px * C + c] = curr[c];
                o->sdesc[rs * npx * C + px * C + c] = intra[c];
            }
            ++o->st_writes;
        }
        if (((size_t)ldraw(o, px) % nLR) == 0) {
            int nx, ny;
            neighbor_pos(ldraw(o, px), 1, &nx, &ny, x, y, LBSP_BORDER, W, H);
            const size_t rs = (size_t)ldraw(o, px) % N;
            const size_t npix = (size_t)ny * W + nx;
            for (size_t c = 0; c < C; ++c) {
                o->scol[rs * npx * C + npix * C + c] = curr[c];
                o->sdesc[rs * npx * C + npix * C + c] = intra[c];
            }
            ++o->st_writes;
        }
    }
    /* :577-580: median blur into the last mask, which is the output; the frame becomes the last colour frame */
    median_binary(o->rawFG, o->lastFG, o->colcnt, W, H, o->p.default_median_blur_kernel_size);
    memcpy(mask, o->lastFG, npx);
    memcpy(o->lastColor, img, npx * C);
    return OSUB_OK;
}

/* BackgroundSubtractorLOBSTER::getBackgroundImage, :583-600: the per-channel float mean of the
 * samples (sum of sample/N in sample order), converted to 8 bits with rounding */
int olob_get_background(const olob_t* o, uint8_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t C = (size_t)o->C, N = o->p.bg_samples, n = o->npx * C;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->scol[s * n + i]) / (float)N;
        out[i] = sat_u8f(acc);
    }
    return OSUB_OK;
}

/* BackgroundSubtractorLOBSTER::getBackgroundDescriptorsImage, :602-620 */
int olob_get_background_descriptors(const olob_t* o, uint16_t* out) {
    if (!o->initialized) return OSUB_ENOTINIT;
    const size_t C = (size_t)o->C, N = o->p.bg_samples, n = o->npx * C;
    for (size_t i = 0; i < n; ++i) {
        float acc = 0.0f;
        for (size_t s = 0; s < N; ++s) acc += ((float)o->sdesc[s * n + i]) / (float)N;
        out[i] = sat_u16f(acc);
    }
    return OSUB_OK;
}

const void* olob_map(const olob_t* o, int which, size_t* nbytes) {
    const size_t npx = o->npx, C = (size_t)o->C, N = o->p.bg_samples;
    size_t n = 0;
    const void* p = NULL;
    switch (which) {
        case OLOB_MAP_LAST_FG: p = o->lastFG; n = npx; break;
        case OLOB_MAP_ROI: p = o->roi; n = npx; break;
        case OLOB_MAP_LAST_COLOR: p = o->lastColor; n = npx * C; break;
        case OLOB_MAP_LAST_DESC: p = o->lastDesc; n = npx * C * 2; break;
        case OLOB_MAP_SAMPLE_COLOR: p = o->scol; n = N * npx * C; break;
        case OLOB_MAP_SAMPLE_DESC: p = o->sdesc; n = N * npx * C * 2; break;
        case OLOB_MAP_LUT: p = o->lut; n = 256; break;
        default: break;
    }
    if (nbytes) *nbytes = o->initialized ? n : 0;
    return o->initialized ? p : NULL;
}

void olob_get_scalars(const olob_t* o, olob_scalars* s) {
    memset(s, 0, sizeof(*s));
    s->frames = o->frames;
    s->n_relevant_px = o->n_rel;
    s->orig_roi_px = o->orig_roi;
    s->stat_samples_evaluated = o->st_samples;
    s->stat_sample_writes = o->st_writes;
}
