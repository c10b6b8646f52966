// Device-side state of the PAWCS path (BackgroundSubtractorPAWCS, one and three channels).
//
// Exactness scheme. The reference scans pixels in raster order; a pixel reads state that earlier
// pixels of the same frame wrote in five ways, and each is resolved explicitly:
//  (1) its own local dictionary, whose last slot an earlier pixel's neighbour update may have
//      replaced: the frame's "local" pass reruns a pixel whose replacement source changed, until
//      no source changes (a fixed point in raster order);
//  (2) the illumination-update mask, set by the pixel on its left: each pixel's outcome is
//      computed for both values of the mask and a per-row scan picks the right one;
//  (3) the global dictionary: only the replaceable word (the last dictionary slot) changes
//      features during a frame, so a sequential scan visits only the items whose outcome depends
//      on it; the spatial maps are then resolved per 2x2 cell (at most four items each) and the
//      word weights by ordered sums;
//  (4) the neighbour's dictionary and raw decision read by a neighbour update: resolved per target
//      pixel over its (at most 24) updaters in raster order;
//  (5) draw indices: every rand() of the reference is draw k of (seed, frame, pixel), and each
//      stage knows how many draws precede it.
// Three channels: the neighbour update edits the target's words themselves (last frame,
// occurrences, descriptor, colour), so (1) becomes "the frame-start dictionary after the loops of
// every earlier updater, applied in raster order by the target's own local pass", a pixel is rerun
// when an earlier updater's loop inputs (target, loop draw start, weight threshold) changed, and the
// loops of later updaters run once the fixed point is reached (pawcs3_kernels.cu).
#pragma once
#include "lvbgs_internal.h"

namespace lvbgs {

constexpr int kPwMaxLocal = 25;   // local words of a one-channel stream (50/2)
constexpr int kPw3MaxLocal = 50;  // local words of a three-channel stream (50)
constexpr int kPwMaxGlobal = 32;  // global words supported (12 / 25 at the default 50 words)
constexpr int kPwGlutStride = 32; // bytes per pixel of the global sort tables
constexpr uint32_t kPwNone = 0xffffffffu;

// frame-level state specific to PAWCS (the common part lives in StreamCtl)
struct PawcsCtl {
    unsigned long long lword_offset;     // m_nLocalWordWeightOffset
    int moving_cam;                      // m_bUsingMovingCamera
    int L, G;                            // m_nCurrLocalWords, m_nCurrGlobalWords
    float last_nonflat_ratio;            // m_fLastNonFlatRegionRatio
    unsigned long long nflat_acc;        // flat pixels of the frame in flight
    unsigned long long ds_roi_count;     // m_nDownSampledROIPxCount
    // global words by pool identity
    unsigned int gw_color[kPwMaxGlobal];
    unsigned int gw_desc[kPwMaxGlobal];   // channels 0 and 1 (16 bits each)
    unsigned int gw_desc2[kPwMaxGlobal];  // channel 2 (three channels)
    unsigned int gw_bits[kPwMaxGlobal];
    float gw_weight[kPwMaxGlobal];
    int gdict[kPwMaxGlobal];             // dictionary slot -> pool word
    int gnext;                           // next unused pool word (initialization)
    // global scan results of the frame in flight
    unsigned int wr_color, wr_desc, wr_desc2, wr_bits;  // replaceable word's features after the frame's items
    unsigned int n_repl;                      // replacements of the replaceable word this frame
    unsigned int n_rounds, n_dirty;           // fixed-point rounds of the frame, dirty pixels left
    unsigned long long st_words, st_events, st_nb;
    float frame_ratio;                   // mean L1 distance ratio of the frame-level analysis
    int reset_pending;                   // automatic reset decided this frame
    int reset_block;                     // the frame entered the reset / camera-motion block (:1479)
    int motion_pending;                  // camera-motion mode switched this frame (refreshModel(1, 1, true))
};

// per-pixel record of the local pass of one frame
struct PwRec {
    float sumW;               // fPotentialLocalWordsWeightSum
    float thrW;               // fLocalWordsWeightSumThreshold
    unsigned long long rate;  // nCurrLocalWordUpdateRate (size_t; SIZE_MAX for an infinite override)
    uint32_t m0, m1;          // final slots illumination-updated when the mask is zero / non-zero
    uint32_t m0hi, m1hi;      // the same for slots 32..63 (three channels)
    uint32_t rsrc;            // replacement source of the own last slot used by the local pass
    uint16_t kScan;           // draw counter after the word scan
    uint16_t incr;            // nCurrWordOccIncr
    uint16_t minColor, minDesc;
    uint8_t flags;            // kRf*
    uint8_t bits;             // popcount of the current descriptor
};
constexpr uint8_t kRfBG = 1, kRfFlat = 2, kRfBorder = 4, kRfU0 = 8, kRfU1 = 16, kRfItem = 32, kRfEvent = 64,
                  kRfRepDraw = 128;

// per-pixel outcome of the global stage / neighbour stage
struct PwOut {
    uint32_t gword;      // matched pool word (kPwNone: none)
    uint32_t epoch;      // replacements of the replaceable word at or before this pixel
    uint32_t q;          // neighbour-update target (kPwNone: no update)
    uint16_t kLoop;      // draw counter at the start of the neighbour loop
    uint8_t segm;        // raw decision (0/255)
    uint8_t gflags;      // bit0 replaced the replaceable word, bit1 contributed to the word weight, bit2 critical
    uint16_t kEnd;       // draw counter after the neighbour loop
    uint8_t rflags;      // neighbour loop: bit0 replaces the target's last word, bit1 reached the last word
    uint8_t chg;         // three channels: the loop inputs (target, kLoop, thrW) changed this round
    float thrW;          // weight threshold of the loop (snapshot of the round's local pass)
    uint32_t qPrev;      // target of the previous round
};

struct PawcsDev {
    StreamDev sd;              // geometry, tiles, frame, mask, float maps, u8 maps, post-processing buffers
    PawcsCtl* pc;
    int L, G, gwW, gwH;
    unsigned int minColor, descOff, nmv;  // m_nMinColorDistThreshold, m_nDescDistThresholdOffset, samples for averages
    float relThr;
    unsigned int lbspOff;
    // local dictionaries, slot-major planes [2][L][npx] by frame parity
    uint8_t* wColor;
    uint16_t* wDesc;
    uint32_t *wOcc, *wFirst, *wLast;
    uint8_t* illum;            // m_oIllumUpdtRegionMask
    uint8_t* unstable;         // m_oUnstableRegionMask
    uint8_t* glut;             // [npx][16] per-pixel global word order (pool indices)
    float* gmap;               // [G][gwW*gwH] spatial occurrence maps, by pool word
    uint16_t* descT;           // current-frame descriptors
    PwRec* rec;
    PwOut* out;
    uint32_t* repBefore;       // latest replacement source before the pixel (kPwNone: none)
    uint32_t* repAfter;        // latest replacement source after the pixel
    uint8_t* uFinal;           // resolved illumination-update bit per pixel
    uint32_t* gitem;           // per pixel: type | fixed word | positions
    float* contrib;            // per pixel: weight contribution to its matched global word (or -1)
    uint8_t* dsRoi;            // down-sampled ROI of the frame-level analysis
    uint8_t* dsFrame;          // down-sampled frame
    uint8_t* uv;               // illumination-update outcomes of the local pass: bit0 mask zero, bit1 non-zero
    uint4* itemList;           // critical global items in raster order, two records each: pixel, colour|bits << 24,
                               // colour threshold|descriptor-bits threshold << 16, descriptors 0-1; descriptor 2|
                               // event flags << 16, fixed position|fixed word << 8, speculative word and epoch
    float* contribList;        // word weight contributions, word-major, raster order within a word
    uint32_t* blkCounts;       // ordered compaction: per block and category counts, then offsets
    uint32_t* catInfo;         // [0..16] category totals, [32..48] category bases
    float* dsAbs;              // |LT - ST| per down-sampled pixel (0 outside the down-sampled ROI)
    uint32_t* updList;         // pixels that update a neighbour this round, raster order
    uint8_t* dirty;            // three channels: pixels whose local pass reruns next round
    uint32_t* gseg;            // global-word scan: per-segment state (pawcs3_kernels.cu)
    uint32_t* gcand;           // global-word scan: candidate items, listed per segment
    uint8_t* gtrue;            // global-word scan: walked candidates that replace the word
};

constexpr int kPwCompactBlk = 1024;  // pixels per block of the ordered compactions
constexpr int kPwCats = kPwMaxGlobal + 1;  // compaction categories: the global words, or the critical items
constexpr int kPwCatBase = 64;       // catInfo: [0, kPwCats) category totals, [kPwCatBase, +kPwCats) bases
constexpr int kPwBootWin = 500;      // BGSPAWCS bootstrap window (frames)

// launch parameters of the PAWCS kernels (a table of streams in device memory)
struct PwParams {
    PawcsDev* streams;
    int nStreams;
    int totalTiles;
    int totalRows;
    int totalCells;
    int round;            // fixed-point round of the local pass (0: every pixel)
    double lr;            // learningRateOverride of the tick (<= 0: internal, inf: never)
    unsigned int* flags;  // [0] dirty pixels of the round, [3] fixed point reached, [4] its round count
    // set for the launches of a fixed-point round: the rounds of a frame are enqueued ahead, and
    // every kernel of a round returns at once when an earlier round reached the fixed point
    const unsigned int* conv;
};
#define PW_ROUND_GUARD(P) \
    if ((P).conv && *(const volatile unsigned int*)(P).conv) return

}  // namespace lvbgs
