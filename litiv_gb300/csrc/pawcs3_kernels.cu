// PAWCS on three-channel (BGR) frames, sm_103a: the kernels whose arithmetic or raster-order
// dependencies differ from the one-channel path (pawcs_kernels.cu). The channel-agnostic stages
// (illumination chain, spatial word maps, neighbour draws, ordered compactions, word weights, global
// word upkeep, post-processing, frame level) are shared.
//
// Reference: modules/video/src/BackgroundSubtractorPAWCS.cpp -- three-channel pixel loop :935-1299
// (local words :1011-1126, global dictionary :1127-1180, neighbour update :1181-1262, feedback
// :1263-1299), refreshModel :107-429, initialize :431-557, frame level :1474-1516, background
// images :1518-1594.
//
// What is different with three channels: the neighbour update edits the target's words themselves
// (last frame and occurrences of the words it matches; descriptor or colour of words it adopts,
// :1205-1247) instead of a copy. So a pixel's dictionary at its turn is its frame-start dictionary
// after the loops of all its earlier updaters, applied in raster order, and those loops depend on
// the updaters' own outcomes. The local pass below applies them itself (from the previous round's
// updater outcomes) before its scan; a pixel is rerun when the loop inputs of an earlier updater in
// its 5x5 window changed (target, loop draw start, weight threshold); the loops of the later
// updaters (including the pixel itself) run once after the fixed point, on the scanned dictionary.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "pawcs_device.cuh"

namespace lvbgs {

// one local word of a three-channel dictionary
struct Pw3Word {
    uint32_t col;   // packed colour
    uint32_t d01;   // descriptors of channels 0 and 1
    uint32_t d2;    // descriptor of channel 2
    uint32_t occ, first, last;
};

__device__ __forceinline__ Pw3Word pw3_load(const PawcsDev& S, int buf, int j, int p) {
    const size_t a = pw_slot(S, buf, j, p);
    const uint8_t* c = S.wColor + a * 3;
    const uint16_t* d = S.wDesc + a * 3;
    Pw3Word w;
    w.col = (uint32_t)c[0] | ((uint32_t)c[1] << 8) | ((uint32_t)c[2] << 16);
    w.d01 = (uint32_t)d[0] | ((uint32_t)d[1] << 16);
    w.d2 = d[2];
    w.occ = S.wOcc[a];
    w.first = S.wFirst[a];
    w.last = S.wLast[a];
    return w;
}
__device__ __forceinline__ void pw3_store(const PawcsDev& S, int buf, int j, int p, const Pw3Word& w) {
    const size_t a = pw_slot(S, buf, j, p);
    uint8_t* c = S.wColor + a * 3;
    uint16_t* d = S.wDesc + a * 3;
    c[0] = (uint8_t)w.col;
    c[1] = (uint8_t)(w.col >> 8);
    c[2] = (uint8_t)(w.col >> 16);
    d[0] = (uint16_t)w.d01;
    d[1] = (uint16_t)(w.d01 >> 16);
    d[2] = (uint16_t)w.d2;
    S.wOcc[a] = w.occ;
    S.wFirst[a] = w.first;
    S.wLast[a] = w.last;
}
__device__ __forceinline__ void pw3_desc(const uint16_t* base, int p, uint32_t& d01, uint32_t& d2) {
    const uint16_t* d = base + (size_t)p * 3;
    d01 = (uint32_t)d[0] | ((uint32_t)d[1] << 16);
    d2 = d[2];
}
__device__ __forceinline__ float pw3_weight(const Pw3Word& w, uint32_t t, unsigned long long off) {
    return pw_weight(w.occ, w.first, w.last, t, off);
}
__device__ __forceinline__ uint32_t pw3_bits(uint32_t d01, uint32_t d2) {
    return (uint32_t)__popc(d01) + (uint32_t)__popc(d2 & 0xffffu);
}
constexpr uint32_t kPw3Flat = 4;  // FLAT_REGION_BIT_COUNT * 2 (three channels)

// what a neighbour update needs of its updater p (all fixed for the frame but thrW and kLoop)
struct Pw3Upd {
    uint32_t col, d01, d2;
    PwThr th;
    int flat;
    unsigned long long rate;
    float thrW;
    uint32_t incr;
    uint32_t p;
};

// the loop inputs of updater p, computed from its frame-start state (the same values its local pass
// computes); its weight threshold comes from the previous round's snapshot (PwOut::thrW, written by
// pw_k_nbr), and its current descriptor from round 0 (a rerun of p in this round rewrites the same
// descriptor)
__device__ __forceinline__ Pw3Upd pw3_updater(const PawcsDev& S, int p, int cur, uint32_t t, double lr) {
    const StreamDev& D = S.sd;
    const float* fm = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
    Pw3Upd u;
    u.p = (uint32_t)p;
    u.col = pw3_color(D.frame, p);
    pw3_desc(S.descT, p, u.d01, u.d2);
    u.flat = pw3_bits(u.d01, u.d2) < kPw3Flat;
    u.th = pw3_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    const int boot = t <= (uint32_t)kBootWin;
    u.incr = (1u + (uint32_t)D.ctl->cooldown) << (u.flat || boot ? 1 : 0);
    if (isinf(lr)) u.rate = ~0ull;
    else if (lr > 0) u.rate = (unsigned long long)ceil(lr);
    else {
        const float T = fm[FM_T * D.npx + p];
        u.rate = u.flat ? (unsigned long long)ceilf(T + kTLower) / 2ull : (unsigned long long)ceilf(T);
    }
    u.thrW = S.out[p].thrW;
    return u;
}

// the neighbour-update loop of updater u over the target's words wd (:1197-1262, three channels: the
// words are edited in place); rawQ is the target's raw decision as the updater sees it, (lq01, lq2)
// its last descriptor; k advances by the loop's draws
__device__ void pw3_loop(Pw3Word* wd, int L, const Pw3Upd& u, int boot, unsigned long long seed, uint32_t t,
                         unsigned long long off, int rawQ, uint32_t lq01, uint32_t lq2, uint32_t& k) {
    const uint32_t nlastDist = pw3_hd(u.d01, u.d2, lq01, lq2);
    const bool nlastFlat = pw3_bits(lq01, lq2) < kPw3Flat;
    float nsum = 0.0f;
    for (int j = 0; j < L && nsum < u.thrW; ++j) {
        Pw3Word& w = wd[j];
        const uint32_t l1 = pw3_l1(u.col, w.col), ncd = pw3_cdist(u.col, w.col);
        const uint32_t ncolorDist = l1 / 2u + ncd * 4u;
        const uint32_t nintra = pw3_hd(u.d01, u.d2, w.d01, w.d2);
        const uint32_t nincr = pw3_bits(w.d01, w.d2) < kPw3Flat ? u.incr * 2u : u.incr;
        if (ncolorDist <= u.th.color && nintra <= u.th.desc) {
            const float nwW = pw3_weight(w, t, off);
            nsum += nwW;
            w.last = t;
            if (nwW < 1.0f) w.occ += nincr;
        } else if (!rawQ && u.flat && (boot || pw_mod(pw_draw(seed, t, u.p, k++), u.rate) == 0u)) {
            if (ncolorDist <= u.th.color && nlastDist <= u.th.desc / 2u) {
                const float nwW = pw3_weight(w, t, off);
                nsum += nwW;
                w.last = t;
                if (nwW < 1.0f) w.occ += nincr;
                w.d01 = u.d01;
                w.d2 = u.d2;
            } else if (nlastFlat && u.flat && nlastDist + nintra <= u.th.desc && ncd <= u.th.color / 4u) {
                const float nwW = pw3_weight(w, t, off);
                nsum += nwW;
                w.last = t;
                if (nwW < 1.0f) w.occ += nincr;
                w.col = u.col;
            }
        }
    }
    if (nsum < 1.0f / (float)off) {
        Pw3Word& w = wd[L - 1];
        w.col = u.col;
        w.d01 = u.d01;
        w.d2 = u.d2;
        w.occ = u.incr;
        w.first = t;
        w.last = t;
    }
}

__device__ void pw3_item_pixel(const PawcsDev& S, int p, const PwRec& R, uint32_t col);

#define PW3_PIXEL_PROLOGUE                                                   \
    const int t0 = blockIdx.x;                                              \
    if (t0 >= P.totalTiles) return;                                         \
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];                \
    const StreamDev& D = S.sd;                                              \
    const int lt = t0 - D.tileBase;                                         \
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;     \
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;

// ------------------------------------------------------------------------------------------
// local pass (:1011-1126): the dictionary at the pixel's turn (frame-start words after its earlier
// updaters' loops, in raster order), then its word scan. Writes the scanned dictionary (next-frame
// buffer; illumination updates as marks) and the record.
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(256, 3) pw3_k_local(PwParams P) {
    PW_ROUND_GUARD(P);
    PW3_PIXEL_PROLOGUE
    if (x >= D.W || y >= D.H) return;
    const int q = y * D.W + x;
    const uint8_t roi = D.roi[q];
    if (!roi) return;
    if (P.round > 0 && !S.dirty[q]) return;
    const StreamCtl* ctl = D.ctl;
    const PawcsCtl* pc = S.pc;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int cur = (int)(ctl->frame_idx & 1ull), nxt = cur ^ 1;
    const int L = S.L;
    const unsigned long long off = pc->lword_offset;
    const int boot = t <= (uint32_t)kBootWin;
    Pw3Word wd[kPw3MaxLocal];
    for (int j = 0; j < L; ++j) wd[j] = pw3_load(S, cur, j, q);
    // earlier updaters' loops (from the previous round's outcomes; none known in round 0)
    if (P.round > 0) {
        uint32_t lq01, lq2;
        pw3_desc(D.lastDesc, q, lq01, lq2);
        for (int dy = -2; dy <= 0; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
                if (dy == 0 && dx >= 0) break;
                const int px = x + dx, py = y + dy;
                if (px < 0 || py < 0 || px >= D.W) continue;
                const int p = py * D.W + px;
                if (!D.roi[p] || S.out[p].q != (uint32_t)q) continue;
                const Pw3Upd u = pw3_updater(S, p, cur, t, P.lr);
                uint32_t k = S.out[p].kLoop;
                pw3_loop(wd, L, u, boot, D.seed, t, off, 0, lq01, lq2, k);
                S.out[p].kEnd = (uint16_t)k;
            }
    }
    // current descriptor (:1003-1010)
    uint8_t taps[3][16];
    pw3_taps(D.frame, D.W, x, y, taps);
    const uint32_t col = pw3_color(D.frame, q);
    uint32_t dsc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const uint32_t v = pw3_ch(col, c);
        dsc[c] = pw_lbsp(taps[c], v, ctl->lut[v]);
    }
    const uint32_t d01 = dsc[0] | (dsc[1] << 16), d2 = dsc[2];
    const uint32_t bits = pw3_bits(d01, d2);
    const int flat = bits < kPw3Flat;
    const int border = roi < 255;
    const float* fm = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
    const float Rr = fm[FM_R * D.npx + q];
    const uint32_t unst = S.unstable[q];
    const PwThr th = pw3_thresholds(Rr, unst, S.minColor, S.descOff);
    const uint32_t incr = (1u + (uint32_t)ctl->cooldown) << (flat || boot ? 1 : 0);
    unsigned long long rate;
    if (isinf(P.lr)) rate = ~0ull;
    else if (P.lr > 0) rate = (unsigned long long)ceil(P.lr);
    else {
        const float T = fm[FM_T * D.npx + q];
        rate = flat ? (unsigned long long)ceilf(T + kTLower) / 2ull : (unsigned long long)ceilf(T);
    }
    uint8_t ord[kPw3MaxLocal];
    for (int j = 0; j < L; ++j) ord[j] = (uint8_t)j;
    const uint32_t lastFG = D.lastFG[q];
    const int moving = pc->moving_cam;
    const float bestW = pw3_weight(wd[0], t, off);
    const float thrW = bestW / (Rr * 2.0f);
    uint32_t k = 0;
    float sumW = 0.0f, lastW = FLT_MAX;
    uint32_t minColor = 765, minDesc = 48;
    unsigned long long mark0 = 0, mark1 = 0, matched = 0;
    int any0 = 0;
    const unsigned long long rateHalf = rate / 2ull + 1ull;
    int i = 0;
    for (; i < L && sumW < thrW; ++i) {
        const Pw3Word& w = wd[i];
        const float cw = pw3_weight(w, t, off);
        const uint32_t l1 = pw3_l1(col, w.col);
        const uint32_t cd = l1 / 2u + pw3_cdist(col, w.col) * 4u;
        const uint32_t intra = pw3_hd(d01, d2, w.d01, w.d2);
        uint32_t inter = 0;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const uint32_t wc = pw3_ch(w.col, c);
            const uint32_t wdc = c == 0 ? (w.d01 & 0xffffu) : c == 1 ? (w.d01 >> 16) : (w.d2 & 0xffffu);
            inter += (uint32_t)__popc(pw_lbsp(taps[c], wc, ctl->lut[wc]) ^ wdc);
        }
        const uint32_t dd = (intra + inter) / 2u;
        if ((!unst || flat || border) && cd <= th.color && l1 >= th.color / 2u && intra <= th.desc / 2u) {
            // illumination update test (:1054): modulus halves (+1) once the mask is non-zero
            const uint32_t r = pw_draw(D.seed, t, (uint32_t)q, k++);
            if (pw_mod(r, rateHalf) == 0u) mark1 |= 1ull << i;
            if (pw_mod(r, any0 ? rateHalf : rate) == 0u) {
                mark0 |= 1ull << i;
                any0 = 1;
            }
        }
        if (dd <= th.desc && cd <= th.color) {
            sumW += cw;
            matched |= 1ull << i;
            minColor = min(minColor, cd);
            minDesc = min(minDesc, dd);
        }
        if (cw > lastW) {
            const uint8_t tmp = ord[i];
            ord[i] = ord[i - 1];
            ord[i - 1] = tmp;
        } else {
            lastW = cw;
        }
    }
    for (; i < L; ++i) {
        const float cw = pw3_weight(wd[i], t, off);
        if (cw > lastW) {
            const uint8_t tmp = ord[i];
            ord[i] = ord[i - 1];
            ord[i - 1] = tmp;
        } else {
            lastW = cw;
        }
    }
    const int bg = sumW >= thrW || border;
    const int occOn = !lastFG || moving;
    unsigned long long m0 = 0, m1 = 0;
    for (int s = 0; s < L; ++s) {
        const int o = ord[s];
        Pw3Word w = wd[o];
        if (matched & (1ull << o)) {
            const float cw = pw3_weight(w, t, off);
            w.last = t;
            if (occOn && cw < 1.0f) w.occ += incr;
        }
        pw3_store(S, nxt, s, q, w);
        if (mark0 & (1ull << o)) m0 |= 1ull << s;
        if (mark1 & (1ull << o)) m1 |= 1ull << s;
    }
    const float initW = 1.0f / (float)off;
    uint8_t flags = (uint8_t)((bg ? kRfBG : 0) | (flat ? kRfFlat : 0) | (border ? kRfBorder : 0) |
                              (mark0 ? kRfU0 : 0) | (mark1 ? kRfU1 : 0));
    if (bg) {
        if (pw_mod(pw_draw(D.seed, t, (uint32_t)q, k), rate) == 0u) {
            flags |= kRfItem | kRfEvent;
            if (pw_mod(pw_draw(D.seed, t, (uint32_t)q, k + 1), rate * 2ull) == 0u) flags |= kRfRepDraw;
        }
    } else {
        if (flat || pw_mod(pw_draw(D.seed, t, (uint32_t)q, k), rate) == 0u) flags |= kRfItem;
        if (sumW < initW) {
            // new local word in the last slot (:1160-1168)
            Pw3Word w;
            w.col = col;
            w.d01 = d01;
            w.d2 = d2;
            w.occ = incr;
            w.first = t;
            w.last = t;
            pw3_store(S, nxt, L - 1, q, w);
        }
    }
    uint16_t* dt = S.descT + (size_t)q * 3;
    dt[0] = (uint16_t)dsc[0];
    dt[1] = (uint16_t)dsc[1];
    dt[2] = (uint16_t)dsc[2];
    S.uv[q] = (uint8_t)((mark0 ? 1 : 0) | (mark1 ? 2 : 0));
    PwRec& R = S.rec[q];
    R.sumW = sumW;
    R.thrW = thrW;
    R.rate = rate;
    R.m0 = (uint32_t)m0;
    R.m1 = (uint32_t)m1;
    R.m0hi = (uint32_t)(m0 >> 32);
    R.m1hi = (uint32_t)(m1 >> 32);
    R.rsrc = kPwNone;
    R.kScan = (uint16_t)k;
    R.incr = (uint16_t)incr;
    R.minColor = (uint16_t)minColor;
    R.minDesc = (uint16_t)minDesc;
    R.flags = flags;
    R.bits = (uint8_t)bits;
    pw3_item_pixel(S, q, R, col);
}

// ------------------------------------------------------------------------------------------
// global items (:1127-1150): as pw_item_pixel with the three-channel match (descriptor bits, then the
// mixed colour distance); run at the end of the pixel's local pass
// ------------------------------------------------------------------------------------------
__device__ void pw3_item_pixel(const PawcsDev& S, int p, const PwRec& R, uint32_t col) {
    const StreamDev& D = S.sd;
    PwOut& O = S.out[p];
    O.gflags = 0;
    O.epoch = 0;
    O.gword = kPwNone;
    if (!(R.flags & kRfItem)) return;
    const PawcsCtl* pc = S.pc;
    const int G = S.G;
    const int wr = pc->gdict[G - 1];
    const float* fm = D.fm + (size_t)(D.ctl->frame_idx & 1ull) * kNumFloatMaps * D.npx;
    const PwThr th = pw3_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    const uint32_t bits = R.bits;
    const uint8_t* lut = S.glut + (size_t)p * kPwGlutStride;
    int fixedPos = G, wrPos = G, fixedWord = -1;
    for (int g = 0; g < G; ++g) {
        const int w = lut[g];
        if (w == wr) {
            wrPos = g;
            continue;
        }
        if (fixedPos == G && pw_absdiff(bits, pc->gw_bits[w]) <= th.desc / 4u && pw3_cmix(col, pc->gw_color[w]) <= th.color) {
            fixedPos = g;
            fixedWord = w;
        }
    }
    const int critical = wrPos < fixedPos;
    if (!critical) O.gword = (uint32_t)fixedWord;
    S.gitem[p] = (uint32_t)(fixedWord < 0 ? 63 : fixedWord) | ((uint32_t)fixedPos << 6) | ((uint32_t)critical << 12);
    if (critical) O.gflags |= 4;
}

// ------------------------------------------------------------------------------------------
// ordered scan of the critical items (:776-786 one channel, :1139-1150 three), segment-parallel. The
// scan's state is only the replaceable word's features (those of its last replacement), only
// candidates (events with the replacement draw and no fixed match) can replace it, and two scans that
// both see an item replace it agree from there on. So each segment of kPw3Seg items is scanned by its
// own warp from kPw3Warm items before its start, from a guessed state (the first of those items'
// features): with replacements frequent, the scan reaches the segment in the true state. One warp
// then walks the segments in order: a segment whose speculative state at its start equals the true
// incoming features keeps its speculative outcomes (one comparison); otherwise its candidates are
// visited up to the first one that replaces the word in both scans. Last, the outcomes: one thread per
// item from the speculative scan, and a warp per walked segment for its walked items.
// Records: two uint4 per item (pixel, colour|bits, thresholds, descriptors 0-1; descriptor 2|event
// flags, fixed position|word, speculative word, speculative epoch | replaced << 31).
// ------------------------------------------------------------------------------------------
constexpr int kPw3Seg = 512;
constexpr int kPw3Warm = 128;
struct Pw3GFeat {
    uint32_t col, d01, d2, bits;
};
struct Pw3Item {
    uint32_t p, col, bits, cthr, dq, d01, d2, fixedPos, fixedWord, specWord, specEpoch;
    bool evRep;
};
__device__ __forceinline__ Pw3Item pw3_item_of(const uint4 a, const uint4 b) {
    Pw3Item it;
    it.p = a.x;
    it.col = a.y & 0xffffffu;
    it.bits = a.y >> 24;
    it.cthr = a.z & 65535u;
    it.dq = a.z >> 16;
    it.d01 = a.w;
    it.d2 = b.x & 65535u;
    it.evRep = ((b.x >> 16) & kRfEvent) && ((b.x >> 16) & kRfRepDraw);
    it.fixedPos = b.y & 255u;
    it.fixedWord = (b.y >> 8) & 255u;
    it.specWord = b.z;
    it.specEpoch = b.w;
    return it;
}
__device__ __forceinline__ Pw3Item pw3_item(const PawcsDev& S, uint32_t i) {
    return pw3_item_of(S.itemList[2 * i], S.itemList[2 * i + 1]);
}
// an item matches the replaceable word: one channel (:776-777) colour distance and descriptor bits;
// three (:1141-1142) descriptor bits and the mixed colour distance
__device__ __forceinline__ bool pw3_gmatch(const Pw3Item& it, const Pw3GFeat& f, bool c3) {
    if (!c3) return pw_absdiff(it.col, f.col) <= it.cthr && pw_absdiff(it.bits, f.bits) <= it.dq;
    return pw_absdiff(it.bits, f.bits) <= it.dq && pw3_cmix(it.col, f.col) <= it.cthr;
}
__device__ __forceinline__ void pw3_set_out(const PawcsDev& S, uint32_t p, uint32_t word, uint32_t epoch, uint32_t repl) {
    PwOut& O = S.out[p];
    O.gword = word;
    O.epoch = epoch;
    O.gflags = (uint8_t)((O.gflags & ~1u) | repl);
}
// per-segment scratch (PawcsDev::gseg, kPw3SegWords words a segment): [0] replacements of the
// speculative scan in the segment, [1..4] its state at the segment's start, [5..8] its state at the
// end, [9] candidates of the segment (listed in gcand from the segment's first item on); from the
// walk: [10] mode (1 kept, 2 walked), [11] true epoch at the segment's start, [12] synchronization
// item (kPwNone: none), [13] epoch shift after it, [14..17] true incoming features
constexpr int kPw3SegWords = 24;
__device__ __forceinline__ uint32_t* pw3_segw(const PawcsDev& S, int s) { return S.gseg + (size_t)s * kPw3SegWords; }
__device__ __forceinline__ bool pw3_is_cand(const Pw3Item& it, int G) { return (int)it.fixedPos >= G && it.evRep; }

// the speculative warp scan of items [a, b) from features f and epoch e, 32 items at a time;
// spec = false: a warm-up (nothing written), true: outcomes into the item records
__device__ void pw3_gscan_range(const PawcsDev& S, int G, int wr, uint32_t a, uint32_t b, Pw3GFeat& f, uint32_t& e,
                                bool spec) {
    const int lane = threadIdx.x & 31;
    const bool c3 = S.sd.C == 3;
    for (uint32_t base = a; base < b; base += 32) {
        const int cnt = (int)min(32u, b - base);
        const bool valid = lane < cnt;
        const Pw3Item it = valid ? pw3_item(S, base + lane) : pw3_item_of(make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0));
        uint32_t myWord = kPwNone, myEpoch = 0, myRepl = 0;
        int cursor = 0;
        while (cursor < cnt) {
            const bool mWr = pw3_gmatch(it, f, c3);
            const bool repl = valid && !mWr && pw3_is_cand(it, G);
            const unsigned cand = __ballot_sync(0xffffffffu, repl && lane >= cursor);
            const int stop = cand ? __ffs(cand) - 1 : cnt;
            if (lane >= cursor && lane < stop) {
                myWord = mWr ? (uint32_t)wr : ((int)it.fixedPos < G ? it.fixedWord : kPwNone);
                myEpoch = e;
            }
            if (stop < cnt) {
                ++e;
                if (lane == stop) {
                    myWord = (uint32_t)wr;
                    myEpoch = e;
                    myRepl = 1;
                }
                f.col = __shfl_sync(0xffffffffu, it.col, stop);
                f.d01 = __shfl_sync(0xffffffffu, it.d01, stop);
                f.d2 = __shfl_sync(0xffffffffu, it.d2, stop);
                f.bits = __shfl_sync(0xffffffffu, it.bits, stop);
            }
            cursor = stop + 1;
        }
        if (spec && valid) {
            uint4& r = S.itemList[2 * (base + lane) + 1];
            r.z = myWord;
            r.w = myEpoch | (myRepl << 31);
        }
    }
}

// phase 1: one warp per segment: its candidates listed, then its speculative scan from a guessed
// state kPw3Warm items before it
extern "C" __global__ void __launch_bounds__(128) pw3_k_gscan_seg(PwParams P) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const uint32_t n = S.catInfo[0];
    const int s = blockIdx.x * 4 + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
    const uint32_t a = (uint32_t)s * kPw3Seg;
    if (a >= n) return;
    const uint32_t b = min(n, a + (uint32_t)kPw3Seg);
    const PawcsCtl* pc = S.pc;
    const int G = S.G;
    const int wr = pc->gdict[G - 1];
    uint32_t* sw = pw3_segw(S, s);
    uint32_t nc = 0;
    for (uint32_t base = a; base < b; base += 32) {
        const bool cand = base + lane < b && pw3_is_cand(pw3_item(S, base + lane), G);
        const unsigned m = __ballot_sync(0xffffffffu, cand);
        if (cand) S.gcand[a + nc + (uint32_t)__popc(m & ((1u << lane) - 1u))] = base + (uint32_t)lane;
        nc += (uint32_t)__popc(m);
    }
    Pw3GFeat f;
    uint32_t e = 0;
    if (a == 0) {
        f.col = pc->gw_color[wr];
        f.d01 = pc->gw_desc[wr];
        f.d2 = pc->gw_desc2[wr];
        f.bits = pc->gw_bits[wr];
    } else {
        const uint32_t w0 = a > (uint32_t)kPw3Warm ? a - (uint32_t)kPw3Warm : 0u;
        const Pw3Item g = pw3_item(S, w0);
        f.col = g.col;
        f.d01 = g.d01;
        f.d2 = g.d2;
        f.bits = g.bits;
        pw3_gscan_range(S, G, wr, w0 + 1, a, f, e, false);
        e = 0;
    }
    if (lane == 0) {
        sw[1] = f.col;
        sw[2] = f.d01;
        sw[3] = f.d2;
        sw[4] = f.bits;
        sw[9] = nc;
    }
    pw3_gscan_range(S, G, wr, a, b, f, e, true);
    if (lane == 0) {
        sw[0] = e;
        sw[5] = f.col;
        sw[6] = f.d01;
        sw[7] = f.d2;
        sw[8] = f.bits;
    }
}

// phase 2: one warp walks the segments in order with the true features. A segment whose speculative
// state at its start equals them is kept; otherwise only its candidates are visited (no other item
// changes the state), up to the first one that replaces the word in both scans, their true outcome
// marked in gtrue
extern "C" __global__ void pw3_k_gscan_walk(PwParams P) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    PawcsCtl* pc = S.pc;
    const int lane = threadIdx.x & 31;
    const uint32_t n = S.catInfo[0];
    const int G = S.G;
    const int wr = pc->gdict[G - 1];
    const bool c3 = S.sd.C == 3;
    Pw3GFeat f;
    f.col = pc->gw_color[wr];
    f.d01 = pc->gw_desc[wr];
    f.d2 = pc->gw_desc2[wr];
    f.bits = pc->gw_bits[wr];
    uint32_t e = 0;
    const int nseg = (int)((n + kPw3Seg - 1) / kPw3Seg);
    for (int s0 = 0; s0 < nseg; s0 += 32) {
        const int sl = s0 + lane;
        uint32_t v[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
        if (sl < nseg) {
            const uint32_t* sw = pw3_segw(S, sl);
#pragma unroll
            for (int j = 0; j < 10; ++j) v[j] = sw[j];
        }
        const int cnt = min(32, nseg - s0);
        for (int k = 0; k < cnt; ++k) {
            const int s = s0 + k;
            uint32_t w[10];
#pragma unroll
            for (int j = 0; j < 10; ++j) w[j] = __shfl_sync(0xffffffffu, v[j], k);
            const Pw3GFeat fin = f;
            const uint32_t ein = e;
            uint32_t mode, sync = kPwNone, offset = 0;
            if (w[1] == f.col && w[2] == f.d01 && w[3] == f.d2 && w[4] == f.bits) {
                mode = 1;  // the speculative scan entered the segment in the true state
                e += w[0];
                f.col = w[5];
                f.d01 = w[6];
                f.d2 = w[7];
                f.bits = w[8];
            } else {
                mode = 2;
                const uint32_t a = (uint32_t)s * kPw3Seg, nc = w[9];
                for (uint32_t base = 0; base < nc && sync == kPwNone; base += 32) {
                    const int cn = (int)min(32u, nc - base);
                    const bool valid = lane < cn;
                    const uint32_t ci = valid ? S.gcand[a + base + lane] : 0u;
                    const Pw3Item it = valid ? pw3_item(S, ci) : pw3_item_of(make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0));
                    uint32_t mine = 0;
                    int cursor = 0, last = cn - 1;
                    while (cursor < cn) {
                        const bool repl = valid && !pw3_gmatch(it, f, c3);
                        const unsigned cm = __ballot_sync(0xffffffffu, repl && lane >= cursor);
                        const int stop = cm ? __ffs(cm) - 1 : cn;
                        if (stop < cn) {
                            ++e;
                            if (lane == stop) mine = 1;
                            f.col = __shfl_sync(0xffffffffu, it.col, stop);
                            f.d01 = __shfl_sync(0xffffffffu, it.d01, stop);
                            f.d2 = __shfl_sync(0xffffffffu, it.d2, stop);
                            f.bits = __shfl_sync(0xffffffffu, it.bits, stop);
                            const uint32_t se = __shfl_sync(0xffffffffu, it.specEpoch, stop);
                            if (se >> 31) {
                                sync = __shfl_sync(0xffffffffu, ci, stop);
                                offset = e - (se & 0x7fffffffu);
                                last = stop;
                                break;
                            }
                        }
                        cursor = stop + 1;
                    }
                    if (valid && lane <= last) S.gtrue[ci] = (uint8_t)mine;
                }
                if (sync != kPwNone) {
                    e = w[0] + offset;
                    f.col = w[5];
                    f.d01 = w[6];
                    f.d2 = w[7];
                    f.bits = w[8];
                }
            }
            if (lane == 0) {
                uint32_t* sw = pw3_segw(S, s);
                sw[10] = mode;
                sw[11] = ein;
                sw[12] = sync;
                sw[13] = offset;
                sw[14] = fin.col;
                sw[15] = fin.d01;
                sw[16] = fin.d2;
                sw[17] = fin.bits;
            }
        }
    }
    if (lane == 0) {
        pc->wr_color = f.col;
        pc->wr_desc = f.d01;
        pc->wr_desc2 = f.d2;
        pc->wr_bits = f.bits;
        pc->n_repl = e;
    }
}

// phase 3a: one thread per item: the kept segments and the items after a synchronization, from the
// speculative scan (epochs shifted); the walked items are left to phase 3b
extern "C" __global__ void __launch_bounds__(256) pw3_k_gscan_fix(PwParams P) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const uint32_t n = S.catInfo[0];
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t* sw = pw3_segw(S, (int)(i / kPw3Seg));
    const uint32_t mode = sw[10], sync = sw[12];
    if (mode == 2 && (sync == kPwNone || i <= sync)) return;
    const uint32_t shift = mode == 1 ? sw[11] : sw[13];
    const Pw3Item it = pw3_item(S, i);
    pw3_set_out(S, it.p, it.specWord, (it.specEpoch & 0x7fffffffu) + shift, it.specEpoch >> 31);
}

// phase 3b: one warp per walked segment, its items up to the synchronization (or all): from the true
// replacers, with warp prefixes of the last replacer and of the replacement count
extern "C" __global__ void __launch_bounds__(128) pw3_k_gscan_fix_walked(PwParams P) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const uint32_t n = S.catInfo[0];
    const int s = blockIdx.x * 4 + (int)(threadIdx.x >> 5), lane = threadIdx.x & 31;
    const uint32_t a = (uint32_t)s * kPw3Seg;
    if (a >= n) return;
    const uint32_t* sw = pw3_segw(S, s);
    if (sw[10] != 2u) return;
    const uint32_t b = min(n, a + (uint32_t)kPw3Seg);
    const uint32_t end = sw[12] == kPwNone ? b : sw[12] + 1;
    const int G = S.G;
    const int wr = S.pc->gdict[G - 1];
    const bool c3 = S.sd.C == 3;
    Pw3GFeat f;
    f.col = sw[14];
    f.d01 = sw[15];
    f.d2 = sw[16];
    f.bits = sw[17];
    uint32_t e = sw[11];
    for (uint32_t base = a; base < end; base += 32) {
        const uint32_t i = base + lane;
        const bool valid = i < end;
        const Pw3Item it = valid ? pw3_item(S, i) : pw3_item_of(make_uint4(0, 0, 0, 0), make_uint4(0, 0, 0, 0));
        const bool rep = valid && pw3_is_cand(it, G) && S.gtrue[i] != 0;
        const unsigned m = __ballot_sync(0xffffffffu, rep);
        const unsigned below = m & ((1u << lane) - 1u);
        Pw3GFeat g = f;
        const int src = below ? 31 - __clz(below) : 0;
        const uint32_t gc = __shfl_sync(0xffffffffu, it.col, src), g01 = __shfl_sync(0xffffffffu, it.d01, src);
        const uint32_t g2 = __shfl_sync(0xffffffffu, it.d2, src), gb = __shfl_sync(0xffffffffu, it.bits, src);
        if (below) {
            g.col = gc;
            g.d01 = g01;
            g.d2 = g2;
            g.bits = gb;
        }
        if (rep) {
            pw3_set_out(S, it.p, (uint32_t)wr, e + (uint32_t)__popc(below) + 1u, 1u);
        } else if (valid) {
            const uint32_t word = pw3_gmatch(it, g, c3) ? (uint32_t)wr : ((int)it.fixedPos < G ? it.fixedWord : kPwNone);
            pw3_set_out(S, it.p, word, e + (uint32_t)__popc(below), 0u);
        }
        if (m) {
            const int top = 31 - __clz(m);
            f.col = __shfl_sync(0xffffffffu, it.col, top);
            f.d01 = __shfl_sync(0xffffffffu, it.d01, top);
            f.d2 = __shfl_sync(0xffffffffu, it.d2, top);
            f.bits = __shfl_sync(0xffffffffu, it.bits, top);
            e += (uint32_t)__popc(m);
        }
    }
}

// pixels rerun next round: an earlier updater in the 5x5 window whose loop inputs changed this
// round and that targets the pixel now or did before
extern "C" __global__ void __launch_bounds__(256) pw3_k_dirty(PwParams P) {
    PW_ROUND_GUARD(P);
    PW3_PIXEL_PROLOGUE
    bool dirty = false;
    if (x < D.W && y < D.H) {
        const int q = y * D.W + x;
        if (D.roi[q]) {
            for (int dy = -2; dy <= 0 && !dirty; ++dy)
                for (int dx = -2; dx <= 2; ++dx) {
                    if (dy == 0 && dx >= 0) break;
                    const int px = x + dx, py = y + dy;
                    if (px < 0 || py < 0 || px >= D.W) continue;
                    const int p = py * D.W + px;
                    if (!D.roi[p]) continue;
                    const PwOut& O = S.out[p];
                    if (O.chg && (O.q == (uint32_t)q || O.qPrev == (uint32_t)q)) {
                        dirty = true;
                        break;
                    }
                }
            S.dirty[q] = dirty ? 1 : 0;
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, dirty);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&P.flags[0], (unsigned)__popc(b));
}

// ------------------------------------------------------------------------------------------
// after the fixed point, per target: the illumination updates of its own scan, then the loops of its
// later updaters (the pixel itself first, when its clamped neighbour position falls back onto it)
// in raster order, on the scanned dictionary; each loop's final draw count goes to its updater
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(256) pw3_k_later(PwParams P) {
    PW3_PIXEL_PROLOGUE
    if (x >= D.W || y >= D.H) return;
    const int q = y * D.W + x;
    if (!D.roi[q]) return;
    const StreamCtl* ctl = D.ctl;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int cur = (int)(ctl->frame_idx & 1ull), nxt = cur ^ 1;
    const int boot = t <= (uint32_t)kBootWin;
    const unsigned long long off = S.pc->lword_offset;
    const int L = S.L;
    const PwRec& R = S.rec[q];
    const uint8_t u = S.uFinal[q];
    const unsigned long long m = (u & 2) ? (((unsigned long long)R.m1hi << 32) | R.m1)
                                         : (((unsigned long long)R.m0hi << 32) | R.m0);
    // any later updater?
    bool any = false;
    for (int dy = 0; dy <= 2 && !any; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
            if (dy == 0 && dx < 0) continue;
            const int px = x + dx, py = y + dy;
            if (px < 0 || px >= D.W || py >= D.H) continue;
            const int p = py * D.W + px;
            if (D.roi[p] && S.out[p].q == (uint32_t)q) {
                any = true;
                break;
            }
        }
    if (!m && !any) return;
    const uint32_t col = pw3_color(D.frame, q);
    uint32_t d01, d2;
    pw3_desc(S.descT, q, d01, d2);
    Pw3Word wd[kPw3MaxLocal];
    for (int j = 0; j < L; ++j) {
        wd[j] = pw3_load(S, nxt, j, q);
        if (m & (1ull << j)) {
            wd[j].col = col;
            wd[j].d01 = d01;
            wd[j].d2 = d2;
        }
    }
    if (any) {
        const int rawQ = S.out[q].segm != 0;
        uint32_t pl01, pl2;
        pw3_desc(D.lastDesc, q, pl01, pl2);
        for (int dy = 0; dy <= 2; ++dy)
            for (int dx = -2; dx <= 2; ++dx) {
                if (dy == 0 && dx < 0) continue;
                const int px = x + dx, py = y + dy;
                if (px < 0 || px >= D.W || py >= D.H) continue;
                const int p = py * D.W + px;
                if (!D.roi[p] || S.out[p].q != (uint32_t)q) continue;
                const Pw3Upd up = pw3_updater(S, p, cur, t, P.lr);
                uint32_t k = S.out[p].kLoop;
                // the target's last descriptor is updated at the end of its own processing (:1290-1293)
                if (p == q) pw3_loop(wd, L, up, boot, D.seed, t, off, rawQ, pl01, pl2, k);
                else pw3_loop(wd, L, up, boot, D.seed, t, off, rawQ, d01, d2, k);
                S.out[p].kEnd = (uint16_t)k;
            }
    }
    for (int j = 0; j < L; ++j) pw3_store(S, nxt, j, q, wd[j]);
}

// ------------------------------------------------------------------------------------------
// commit (:1263-1299): feedback maps, illumination mask, last colour and descriptor, raw mask and
// draw counters (the dictionaries are final after pw3_k_later)
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(256) pw3_k_commit(PwParams P) {
    PW3_PIXEL_PROLOGUE
    const bool in = x < D.W && y < D.H;
    const int p = in ? y * D.W + x : 0;
    const bool act = in && D.roi[p];
    int flat = 0;
    if (act) {
        const StreamCtl* ctl = D.ctl;
        const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
        const int cur = (int)(ctl->frame_idx & 1ull), nxt = cur ^ 1;
        const int boot = t <= (uint32_t)kBootWin;
        const PwRec& R = S.rec[p];
        const PwOut& O = S.out[p];
        flat = (R.flags & kRfFlat) != 0;
        const uint8_t u = S.uFinal[p];
        // the neighbours' updates write 1 & ROI (:1025-1026): 0 in the ROI's edge band of 128
        const int roiBit = D.roi[p] & 1;
        const int uRight = (x + 1 < D.W && D.roi[p + 1]) ? (S.uFinal[p + 1] & 1) : 0;
        const int mStart = (x > 0 && D.roi[p - 1] && (S.uFinal[p - 1] & 1)) ? roiBit : (int)S.illum[p];
        int mEnd;
        if (uRight) mEnd = roiBit;
        else if (u & 1) mEnd = 1;
        else mEnd = mStart > 0 ? mStart - 1 : 0;
        S.illum[p] = (uint8_t)mEnd;
        float fLT, fST;
        pw_factors(t, (int)S.nmv, &fLT, &fST);
        const float* fc = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
        float* fn = D.fm + (size_t)nxt * kNumFloatMaps * D.npx;
        const int npx = D.npx;
        float dLT = fc[FM_DMIN_LT * npx + p], dST = fc[FM_DMIN_ST * npx + p];
        float rLT = fc[FM_RAW_LT * npx + p], rST = fc[FM_RAW_ST * npx + p];
        const float nmc = (float)R.minColor / 765.0f, nmd = (float)R.minDesc / 48.0f;
        const float nd0 = (nmc < nmd) ? nmd : nmc;
        if (R.flags & kRfBG) {
            dLT = dLT * (1.0f - fLT) + nd0 * fLT;
            dST = dST * (1.0f - fST) + nd0 * fST;
            rLT = rLT * (1.0f - fLT);
            rST = rST * (1.0f - fST);
        } else {
            const float qq = (R.thrW - R.sumW) / R.thrW;
            const float nd = (nd0 < qq) ? qq : nd0;
            dLT = dLT * (1.0f - fLT) + nd * fLT;
            dST = dST * (1.0f - fST) + nd * fST;
            rLT = rLT * (1.0f - fLT) + fLT;
            rST = rST * (1.0f - fST) + fST;
        }
        float Rr = fc[FM_R * npx + p], V = fc[FM_V * npx + p], T = fc[FM_T * npx + p];
        const float finLT = fc[FM_FIN_LT * npx + p], finST = fc[FM_FIN_ST * npx + p];
        S.unstable[p] = (Rr > kUnstR || (rLT - finLT) > kUnstRatio || (rST - finST) > kUnstRatio) ? 1 : 0;
        const uint32_t lastFG = D.lastFG[p];
        const float dmin = (dST < dLT) ? dST : dLT, dmax = (dLT < dST) ? dST : dLT;
        if (lastFG || (dmin < kUnstRatio && O.segm)) {
            const float a = T + kTIncr / (dmax * V);
            T = (kTUpper < a) ? kTUpper : a;
        } else {
            const float a = T - kTDecr * V / dmax;
            T = (a < kTLower) ? kTLower : a;
        }
        if (dmax > kUnstRatio && D.blinks[p]) {
            V += boot ? kVIncr * 2 : kVIncr;
        } else {
            const float a = V - kVDecr * ((boot || flat) ? 2.0f : lastFG ? 0.5f : 1.0f);
            V = (a < kVDecr) ? kVDecr : a;
        }
        const float xb = 1.0f + dmin * 2.0f;
        const float hi = xb * xb, lo = __fmaf_rn(xb, xb, -hi);
        if (Rr < hi || (Rr == hi && lo > 0.0f)) {
            Rr += kRVar * (V - kVDecr);
        } else {
            const float a = Rr - kRVar / V;
            Rr = (a < 1.0f) ? 1.0f : a;
        }
        fn[FM_R * npx + p] = Rr;
        fn[FM_V * npx + p] = V;
        fn[FM_T * npx + p] = T;
        fn[FM_DMIN_LT * npx + p] = dLT;
        fn[FM_DMIN_ST * npx + p] = dST;
        fn[FM_RAW_LT * npx + p] = rLT;
        fn[FM_RAW_ST * npx + p] = rST;
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            D.lastCol[(size_t)p * 3 + c] = D.frame[(size_t)p * 3 + c];
            D.lastDesc[(size_t)p * 3 + c] = S.descT[(size_t)p * 3 + c];
        }
        D.intent[p] = O.segm ? (kInValid | kInFG) : kInValid;
        D.kctr[p] = O.q != kPwNone ? O.kEnd : O.kLoop;
    } else if (in) {
        D.intent[p] = 0u;
    }
    const unsigned b = __ballot_sync(0xffffffffu, act && flat);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&S.pc->nflat_acc, (unsigned long long)__popc(b));
}

// ------------------------------------------------------------------------------------------
// frame level, three channels
// ------------------------------------------------------------------------------------------
// down-sampled frame per channel (INTER_AREA, integral scale), its rolling averages and the
// per-pixel L1 |LT - ST| over the channels (:1475-1478)
extern "C" __global__ void pw3_k_ds(PwParams P) {
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const int nds = D.dsW * D.dsH;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nds) return;
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    float fLT, fST;
    pw_factors(t, (int)S.nmv, &fLT, &fST);
    const int bx = i % D.dsW, by = i / D.dsW;
    float e = 0.0f;
    for (int c = 0; c < 3; ++c) {
        const uint8_t* fr = D.frame;
        const int W = D.W;
        const uint8_t vb = area_resample(D.W, D.H, D.dsW, D.dsH, bx, by,
                                         [&](int sx, int sy) { return (int)fr[((size_t)sy * W + sx) * 3 + c]; });
        const size_t k = (size_t)i * 3 + c;
        const float lt = (float)vb * fLT + D.dsLT[k] * (1.0f - fLT);
        const float st = (float)vb * fST + D.dsST[k] * (1.0f - fST);
        D.dsLT[k] = lt;
        D.dsST[k] = st;
        S.dsFrame[k] = vb;
        e = e + fabsf(lt - st);
    }
    S.dsAbs[i] = S.dsRoi[i] ? e : 0.0f;
}

// camera-motion comparison (:1480-1501), three channels: the background image of the words of buffer
// buf, area-down-sampled, against the long-term means: L1 over the channels into dsAbs and the float
// colour distortion (lv::cdist<3>, math.hpp:499-527) into contrib; 0 outside the fully covered blocks
extern "C" __global__ void pw3_k_motion_bg(PwParams P, int buf) {
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const int nds = D.dsW * D.dsH;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nds) return;
    if (S.dsRoi[i] != 255) {
        S.dsAbs[i] = 0.0f;
        S.contrib[i] = 0.0f;
        return;
    }
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    const unsigned long long off = S.pc->lword_offset;
    const int bx = i % D.dsW, by = i / D.dsW;
    float a[3], b[3], e = 0.0f;
    for (int c = 0; c < 3; ++c) {
        // channel c of the background image (0 outside the ROI), area-down-sampled
        b[c] = (float)area_resample(D.W, D.H, D.dsW, D.dsH, bx, by, [&](int sx, int sy) {
            const int p = sy * D.W + sx;
            if (!D.roi[p]) return 0;
            float tw = 0.0f, tc = 0.0f;
            for (int j = 0; j < S.L; ++j) {
                const size_t a = pw_slot(S, buf, j, p);
                const float w = pw_weight(S.wOcc[a], S.wFirst[a], S.wLast[a], t, off);
                tc = tc + (float)S.wColor[a * 3 + c] * w;
                tw = tw + w;
            }
            const int r = __float2int_rn(tc / tw);
            return r < 0 ? 0 : r > 255 ? 255 : r;
        });
        a[c] = D.dsLT[(size_t)i * 3 + c];
        e = e + fabsf(a[c] - b[c]);
    }
    S.dsAbs[i] = e;
    bool nonconst = false, nonnull = a[0] != b[0];
    for (int c = 1; c < 3; ++c) {
        nonconst = nonconst || a[c] != a[c - 1] || b[c] != b[c - 1];
        nonnull = nonnull || a[c] != b[c];
    }
    float cd = 0.0f;
    if (nonconst && nonnull) {
        float cs = 0.0f, bs = 0.0f, mx = 0.0f;
        for (int c = 0; c < 3; ++c) {
            cs = cs + a[c] * a[c];
            bs = bs + b[c] * b[c];
            mx = mx + a[c] * b[c];
        }
        bs = bs + FLT_EPSILON;
        const float r = (mx * mx) / bs;
        if (!(cs <= r)) cd = __fsqrt_rn(cs - r);
    }
    S.contrib[i] = cd;
}

// ------------------------------------------------------------------------------------------
// refreshModel (:107-429), three channels
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(128) pw3_k_refresh_local(PawcsDev S, uint32_t t, int buf, int baseOcc,
                                                                       float decr, int force, int onlyPending,
                                                                       int useDil) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const StreamDev& D = S.sd;
    if (p >= D.npx) return;
    if (onlyPending && S.pc->reset_pending == 0) return;
    if (!D.roi[p]) return;
    if (!(force || !useDil || D.dilInv[p] != 0)) return;
    const int L = S.L;
    const int x0 = p % D.W, y0 = p / D.W;
    const unsigned long long off = S.pc->lword_offset;
    const float* fm = D.fm + (size_t)buf * kNumFloatMaps * D.npx;
    const PwThr th = pw3_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    Pw3Word wd[kPw3MaxLocal];
    for (int j = 0; j < L; ++j) wd[j] = pw3_load(S, buf, j, p);
    if (decr > 0.0f)
        for (int j = 0; j < L; ++j)
            if (wd[j].first != kPwNone) wd[j].occ -= (uint32_t)(decr * (float)wd[j].occ);
    uint32_t k = D.kctr[p];
    for (int it = 0; it < 98; ++it) {
        const uint32_t r = pw_draw(D.seed, t, (uint32_t)p, k++);
        int rr = 1 + (int)(r % 512u), xx = 0, yy = 0;
        for (int c = 0; c < 49; ++c) {
            rr -= pw_pat7[c];
            if (rr <= 0) {
                xx = c % 7;
                yy = c / 7;
                break;
            }
        }
        int sx = x0 + xx - 3, sy = y0 + yy - 3;
        sx = sx < 2 ? 2 : sx >= D.W - 2 ? D.W - 3 : sx;
        sy = sy < 2 ? 2 : sy >= D.H - 2 ? D.H - 3 : sy;
        const int sp = sy * D.W + sx;
        if (!(force || !useDil || D.dilInv[sp] != 0)) continue;
        const uint32_t scol = pw3_color(D.lastCol, sp);
        uint32_t s01, s2;
        pw3_desc(D.lastDesc, sp, s01, s2);
        int i;
        for (i = 0; i < L; ++i) {
            if (wd[i].first == kPwNone) continue;
            if (pw3_cmix(scol, wd[i].col) <= th.color && pw3_hd(s01, s2, wd[i].d01, wd[i].d2) <= th.desc) {
                wd[i].occ += 1;
                wd[i].last = t;
                break;
            }
        }
        if (i == L) {
            i = L - 1;
            wd[i].col = scol;
            wd[i].d01 = s01;
            wd[i].d2 = s2;
            wd[i].occ = (uint32_t)baseOcc;
            wd[i].first = t;
            wd[i].last = t;
        }
        while (i > 0 && (wd[i - 1].first == kPwNone || pw3_weight(wd[i], t, off) > pw3_weight(wd[i - 1], t, off))) {
            const Pw3Word tmp = wd[i];
            wd[i] = wd[i - 1];
            wd[i - 1] = tmp;
            --i;
        }
    }
    for (int i = 1; i < L; ++i) {
        if (wd[i].first != kPwNone) continue;
        const int ri = (int)(pw_draw(D.seed, t, (uint32_t)p, k++) % (uint32_t)i);
        const int offc = (int)(pw_draw(D.seed, t, (uint32_t)p, k++) % (th.color / 3u + 1u)) - (int)(th.color / 6u);
        uint32_t col = 0;
        for (int c = 0; c < 3; ++c) {
            const int v = (int)pw3_ch(wd[ri].col, c) + offc;
            col |= (uint32_t)(v < 0 ? 0 : v > 255 ? 255 : v) << (8 * c);
        }
        wd[i].col = col;
        wd[i].d01 = wd[ri].d01;
        wd[i].d2 = wd[ri].d2;
        const uint32_t occ = (uint32_t)((float)wd[ri].occ * ((float)(L - i) / (float)L));
        wd[i].occ = occ > 1u ? occ : 1u;
        wd[i].first = t;
        wd[i].last = t;
    }
    for (int j = 0; j < L; ++j) pw3_store(S, buf, j, p, wd[j]);
    D.kctr[p] = (uint16_t)k;
}

extern "C" __global__ void pw3_k_refresh_global(PawcsDev S, uint32_t t, int buf, int force, int onlyPending,
                                                int useDil) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    PawcsCtl* pc = S.pc;
    if (onlyPending && pc->reset_pending == 0) return;
    const StreamDev& D = S.sd;
    const int G = S.G;
    const size_t n = (size_t)S.gwW * S.gwH;
    const unsigned long long off = pc->lword_offset;
    const float* fm = D.fm + (size_t)buf * kNumFloatMaps * D.npx;
    size_t incr = (size_t)D.npx / (size_t)G > 1 ? (size_t)D.npx / (size_t)G : 1;
    for (int pass = 0; pass < 2; ++pass) {
        for (size_t p = 0; p < (size_t)D.npx; p += incr) {
            if (!D.roi[p]) continue;
            if (!(force || !useDil || D.dilInv[p] != 0)) continue;
            const int x = (int)(p % D.W), y = (int)(p / D.W);
            const size_t cidx = (size_t)(y / 2) * S.gwW + (x / 2);
            const PwThr th = pw3_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
            const Pw3Word best = pw3_load(S, buf, 0, (int)p);
            const float bw = pw3_weight(best, t, off);
            const uint32_t bb = pw3_bits(best.d01, best.d2);
            int uninit = 0, g;
            for (g = 0; g < G; ++g) {
                const int w = pc->gdict[g];
                if (w < 0) {
                    uninit = 1;
                    continue;
                }
                if (pw_absdiff(bb, pc->gw_bits[w]) <= th.desc / 4u && pw3_cmix(best.col, pc->gw_color[w]) <= th.color) break;
            }
            if (g == G) {
                g = G - 1;
                const int w = uninit ? pc->gnext++ : pc->gdict[g];
                pc->gw_color[w] = best.col;
                pc->gw_desc[w] = best.d01;
                pc->gw_desc2[w] = best.d2;
                pc->gw_bits[w] = bb;
                for (size_t i = 0; i < n; ++i) S.gmap[(size_t)w * n + i] = 0.0f;
                pc->gw_weight[w] = 0.0f;
                pc->gdict[g] = w;
            }
            const int w = pc->gdict[g];
            float* lw = S.gmap + (size_t)w * n + cidx;
            if (*lw < bw) {
                pc->gw_weight[w] = pc->gw_weight[w] + bw;
                *lw = *lw + bw;
            }
            while (g > 0 && (pc->gdict[g - 1] < 0 || pc->gw_weight[pc->gdict[g]] > pc->gw_weight[pc->gdict[g - 1]])) {
                const int tmp = pc->gdict[g];
                pc->gdict[g] = pc->gdict[g - 1];
                pc->gdict[g - 1] = tmp;
                --g;
            }
        }
        incr = incr / 3 > 1 ? incr / 3 : 1;
    }
    for (int g = 0; g < G; ++g) {
        if (pc->gdict[g] >= 0) continue;
        const int w = pc->gnext++;
        pc->gw_color[w] = 0;
        pc->gw_desc[w] = 0;
        pc->gw_desc2[w] = 0;
        pc->gw_bits[w] = 0;
        for (size_t i = 0; i < n; ++i) S.gmap[(size_t)w * n + i] = 0.0f;
        pc->gw_weight[w] = 0.0f;
        pc->gdict[g] = w;
    }
}

// initial state (:472-520) of the three-channel word planes; the maps as pw_k_init
extern "C" __global__ void pw3_k_init(PawcsDev S) {
    const StreamDev& D = S.sd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        for (int b = 0; b < 2; ++b) {
            float* f = D.fm + (size_t)b * kNumFloatMaps * D.npx;
            for (int m = 0; m < kNumFloatMaps; ++m) f[m * D.npx + p] = 0.0f;
            f[FM_T * D.npx + p] = kTLower;
            f[FM_R * D.npx + p] = 2.0f;
            f[FM_V * D.npx + p] = kVIncr * 10;
            Pw3Word w;
            w.col = 0;
            w.d01 = 0;
            w.d2 = 0;
            w.occ = 0;
            w.first = kPwNone;
            w.last = 0;
            for (int j = 0; j < S.L; ++j) pw3_store(S, b, j, p, w);
        }
        S.illum[p] = 0;
        S.unstable[p] = 0;
        D.blinks[p] = 0;
        D.lastRawFG[p] = 0;
        D.lastFG[p] = 0;
        D.dilInv[p] = 0;
        D.lastRawBlink[p] = 0;
        D.kctr[p] = 0;
        for (int g = 0; g < kPwGlutStride; ++g) S.glut[(size_t)p * kPwGlutStride + g] = (uint8_t)g;
    }
}

// last colour and LBSP descriptors of the initialization frame, per channel (descriptors strictly
// inside the 2-pixel border)
extern "C" __global__ void pw3_k_init_last(PawcsDev S, const uint8_t* img) {
    const StreamDev& D = S.sd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        const int x = p % D.W, y = p / D.W;
        uint8_t c[3] = {0, 0, 0};
        uint16_t d[3] = {0, 0, 0};
        if (D.roi[p]) {
            for (int k = 0; k < 3; ++k) c[k] = img[(size_t)p * 3 + k];
            if (x > 2 && y > 2 && x < D.W - 2 && y < D.H - 2) {
                uint8_t taps[3][16];
                pw3_taps(img, D.W, x, y, taps);
                for (int k = 0; k < 3; ++k) d[k] = (uint16_t)pw_lbsp(taps[k], c[k], D.ctl->lut[c[k]]);
            }
        }
        for (int k = 0; k < 3; ++k) {
            D.lastCol[(size_t)p * 3 + k] = c[k];
            D.lastDesc[(size_t)p * 3 + k] = d[k];
        }
    }
}

// background image / descriptors (:1518-1594), three channels
extern "C" __global__ void pw3_k_background(PawcsDev S, int buf, uint8_t* outCol, uint16_t* outDesc) {
    const StreamDev& D = S.sd;
    const uint32_t t = (uint32_t)D.ctl->frame_idx;
    const unsigned long long off = S.pc->lword_offset;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        if (!D.roi[p]) {
            for (int c = 0; c < 3; ++c) {
                if (outCol) outCol[(size_t)p * 3 + c] = 0;
                if (outDesc) outDesc[(size_t)p * 3 + c] = 0;
            }
            continue;
        }
        float tw = 0.0f, tc[3] = {0.0f, 0.0f, 0.0f}, td[3] = {0.0f, 0.0f, 0.0f};
        for (int j = 0; j < S.L; ++j) {
            const size_t a = pw_slot(S, buf, j, p);
            const float w = pw_weight(S.wOcc[a], S.wFirst[a], S.wLast[a], t, off);
            for (int c = 0; c < 3; ++c) {
                tc[c] = tc[c] + (float)S.wColor[a * 3 + c] * w;
                td[c] = td[c] + (float)S.wDesc[a * 3 + c] * w;
            }
            tw = tw + w;
        }
        for (int c = 0; c < 3; ++c) {
            if (outCol) {
                const int r = __float2int_rn(tc[c] / tw);
                outCol[(size_t)p * 3 + c] = (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
            }
            if (outDesc) {
                const int r = __float2int_rn(td[c] / tw);
                outDesc[(size_t)p * 3 + c] = (uint16_t)(r < 0 ? 0 : r > 65535 ? 65535 : r);
            }
        }
    }
}

}  // namespace lvbgs
