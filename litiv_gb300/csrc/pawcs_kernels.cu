// PAWCS (BackgroundSubtractorPAWCS, one channel) on sm_103a: the frame step as parallel passes that
// reproduce the reference's sequential raster scan exactly (scheme in pawcs_internal.h).
//
// Reference: modules/video/src/BackgroundSubtractorPAWCS.cpp -- refreshModel :107-429, initialize
// :431-557, apply :559-1516 (one-channel pixel loop :608-934, global words :1300-1334,
// post-processing :1443-1461, frame level :1462-1516), word weights :1596-1602.
#include <cuda_runtime.h>
#include <float.h>
#include <stdint.h>

#include "pawcs_device.cuh"

namespace lvbgs {

// the neighbour-update loop of updater p over target q's words (:850-878, one channel: the
// reference updates a copy of each word, so only the weight sum and the draws matter); returns
// the replacement decision and the pixel's draw count after the loop
struct PwWordSrc {
    const PawcsDev* S;
    int q, buf, L;
    uint32_t m;        // words whose colour/descriptor are the target's current values (illumination)
    uint32_t qcol, qdesc;
    int repl;          // last slot replaced by source rsrc
    uint32_t rcol, rdesc, rincr, t;
};
__device__ __forceinline__ void pw_word(const PwWordSrc& s, int j, uint32_t& c, uint32_t& d, uint32_t& o, uint32_t& f,
                                        uint32_t& l) {
    if (s.repl && j == s.L - 1) {
        c = s.rcol;
        d = s.rdesc;
        o = s.rincr;
        f = s.t;
        l = s.t;
        return;
    }
    const size_t a = pw_slot(*s.S, s.buf, j, s.q);
    c = s.S->wColor[a];
    d = s.S->wDesc[a];
    o = s.S->wOcc[a];
    f = s.S->wFirst[a];
    l = s.S->wLast[a];
    if (s.m & (1u << j)) {
        c = s.qcol;
        d = s.qdesc;
    }
}

// ------------------------------------------------------------------------------------------
// local pass: the pixel's word scan (:632-748) against its dictionary at its turn -- the frame-start
// dictionary with the last slot replaced by the latest earlier neighbour update, if any. Writes the
// scanned dictionary (next-frame buffer, illumination updates not yet applied) and the record.
// ------------------------------------------------------------------------------------------
__device__ void pw_item_pixel(const PawcsDev& S, int p, const PwRec& R, uint32_t col);

extern "C" __global__ void __launch_bounds__(256) pw_k_local(PwParams P) {
    PW_ROUND_GUARD(P);
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
    if (x >= D.W || y >= D.H) return;
    const int p = y * D.W + x;
    const uint8_t roi = D.roi[p];
    if (!roi) return;
    PwRec& R = S.rec[p];
    const uint32_t rsrc = S.repBefore[p];
    if (P.round > 0 && R.rsrc == rsrc) return;  // inputs unchanged since its last local pass
    const StreamCtl* ctl = D.ctl;
    const PawcsCtl* pc = S.pc;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int cur = (int)(ctl->frame_idx & 1ull), nxt = cur ^ 1;
    const int L = S.L;
    const unsigned long long off = pc->lword_offset;
    const int boot = t <= (uint32_t)kBootWin;
    // current descriptor
    uint8_t taps[16];
    pw_taps(D.frame, D.W, x, y, taps);
    const uint32_t col = D.frame[p];
    const uint32_t desc = pw_lbsp(taps, col, ctl->lut[col]);
    const uint32_t bits = __popc(desc);
    const int flat = bits < 2u;
    const int border = roi < 255;
    const float* fm = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
    const float Rr = fm[FM_R * D.npx + p];
    const uint32_t unst = S.unstable[p];
    const PwThr th = pw_thresholds(Rr, unst, S.minColor, S.descOff);
    const uint32_t cooldown = (uint32_t)ctl->cooldown;
    const uint32_t incr = (1u + cooldown) << (flat || boot ? 1 : 0);
    unsigned long long rate;
    if (isinf(P.lr)) rate = ~0ull;
    else if (P.lr > 0) rate = (unsigned long long)ceil(P.lr);
    else {
        const float T = fm[FM_T * D.npx + p];
        rate = flat ? (unsigned long long)ceilf(T + kTLower) / 2ull : (unsigned long long)ceilf(T);
    }
    // the dictionary at the pixel's turn: the frame-start words (read-only in this pass), the last
    // one replaced by an earlier neighbour update (its colour and descriptor, occurrences = its incr)
    PwWordSrc ws;
    ws.S = &S;
    ws.q = p;
    ws.buf = cur;
    ws.L = L;
    ws.m = 0;
    ws.repl = rsrc != kPwNone;
    ws.t = t;
    if (ws.repl) {
        ws.rcol = D.frame[rsrc];
        ws.rdesc = S.descT[rsrc];
        ws.rincr = S.rec[rsrc].incr;
    }
    uint8_t ord[kPwMaxLocal];
    for (int j = 0; j < L; ++j) ord[j] = (uint8_t)j;
    const uint32_t lastFG = D.lastFG[p];
    const int moving = pc->moving_cam;
    uint32_t c0, d0, o0, f0, l0;
    pw_word(ws, 0, c0, d0, o0, f0, l0);
    const float bestW = pw_weight(o0, f0, l0, t, off);
    const float thrW = bestW / (Rr * 2.0f);
    // word scan with one bubble pass
    uint32_t k = 0;
    float sumW = 0.0f, lastW = FLT_MAX;
    uint32_t minColor = 255, minDesc = 16;
    uint32_t mark0 = 0, mark1 = 0, matched = 0;
    int any0 = 0;
    const unsigned long long rateHalf = rate / 2ull + 1ull;
    int i = 0;
    for (; i < L && sumW < thrW; ++i) {
        uint32_t wci, wdi, woi, wfi, wli;
        pw_word(ws, i, wci, wdi, woi, wfi, wli);
        const float w = pw_weight(woi, wfi, wli, t, off);
        const uint32_t cd = pw_absdiff(col, wci);
        const uint32_t intra = __popc(desc ^ wdi);
        const uint32_t inter = __popc(pw_lbsp(taps, wci, ctl->lut[wci]) ^ wdi);
        const uint32_t dd = (intra + inter) / 2u;
        if ((!unst || flat || border) && cd <= th.color && cd >= th.color / 2u && intra <= th.desc / 2u) {
            // illumination update test (:684): modulus halves (+1) once the mask is non-zero
            const uint32_t r = pw_draw(D.seed, t, (uint32_t)p, k++);
            if (pw_mod(r, rateHalf) == 0u) mark1 |= 1u << i;
            if (pw_mod(r, any0 ? rateHalf : rate) == 0u) {
                mark0 |= 1u << i;
                any0 = 1;
            }
        }
        if (dd <= th.desc && cd <= th.color) {
            sumW += w;
            matched |= 1u << i;
            minColor = min(minColor, cd);
            minDesc = min(minDesc, dd);
        }
        if (w > lastW) {
            const uint8_t tmp = ord[i];
            ord[i] = ord[i - 1];
            ord[i - 1] = tmp;
        } else {
            lastW = w;
        }
    }
    for (; i < L; ++i) {
        uint32_t wci, wdi, woi, wfi, wli;
        pw_word(ws, i, wci, wdi, woi, wfi, wli);
        const float w = pw_weight(woi, wfi, wli, t, off);
        if (w > lastW) {
            const uint8_t tmp = ord[i];
            ord[i] = ord[i - 1];
            ord[i - 1] = tmp;
        } else {
            lastW = w;
        }
    }
    const int bg = sumW >= thrW || border;
    // the scanned dictionary in its new order: matched words seen now, occurrences incremented
    const int occOn = !lastFG || moving;
    uint32_t m0 = 0, m1 = 0;
    for (int s = 0; s < L; ++s) {
        const int o = ord[s];
        uint32_t wco, wdo, woo, wfo, wlo;
        pw_word(ws, o, wco, wdo, woo, wfo, wlo);
        uint32_t occ = woo, last = wlo;
        if (matched & (1u << o)) {
            last = t;
            if (occOn && pw_weight(woo, wfo, wlo, t, off) < 1.0f) occ += incr;
        }
        const size_t d = pw_slot(S, nxt, s, p);
        S.wColor[d] = (uint8_t)wco;
        S.wDesc[d] = (uint16_t)wdo;
        S.wOcc[d] = occ;
        S.wFirst[d] = wfo;
        S.wLast[d] = last;
        if (mark0 & (1u << o)) m0 |= 1u << s;
        if (mark1 & (1u << o)) m1 |= 1u << s;
    }
    const float initW = 1.0f / (float)off;
    uint8_t flags = (uint8_t)((bg ? kRfBG : 0) | (flat ? kRfFlat : 0) | (border ? kRfBorder : 0) |
                              (mark0 ? kRfU0 : 0) | (mark1 ? kRfU1 : 0));
    if (bg) {
        // global dictionary event (:774) and, when nothing matches, the replacement draw (:785)
        if (pw_mod(pw_draw(D.seed, t, (uint32_t)p, k), rate) == 0u) {
            flags |= kRfItem | kRfEvent;
            if (pw_mod(pw_draw(D.seed, t, (uint32_t)p, k + 1), rate * 2ull) == 0u) flags |= kRfRepDraw;
        }
    } else {
        if (flat || pw_mod(pw_draw(D.seed, t, (uint32_t)p, k), rate) == 0u) flags |= kRfItem;
        if (sumW < initW) {
            // new local word in the last slot (:822-830)
            const size_t d = pw_slot(S, nxt, L - 1, p);
            S.wColor[d] = (uint8_t)col;
            S.wDesc[d] = (uint16_t)desc;
            S.wOcc[d] = incr;
            S.wFirst[d] = t;
            S.wLast[d] = t;
        }
    }
    S.descT[p] = (uint16_t)desc;
    S.uv[p] = (uint8_t)((mark0 ? 1 : 0) | (mark1 ? 2 : 0));
    R.sumW = sumW;
    R.thrW = thrW;
    R.rate = rate;
    R.m0 = m0;
    R.m1 = m1;
    R.rsrc = rsrc;
    R.kScan = (uint16_t)k;
    R.incr = (uint16_t)incr;
    R.minColor = (uint16_t)minColor;
    R.minDesc = (uint16_t)minDesc;
    R.m0hi = 0;
    R.m1hi = 0;
    R.flags = flags;
    R.bits = (uint8_t)bits;
    pw_item_pixel(S, p, R, col);
}

// ------------------------------------------------------------------------------------------
// illumination chain: the mask a pixel sees is 1 & ROI when its left neighbour made an illumination
// update this frame (the neighbour writes 1 & m_oROI, :689-690: 1 inside the ROI, 0 in its edge band
// of 128), else its frame-start value (:686-688, :893-894). Each pixel's outcome is a function of its
// left neighbour's (two states), so one warp per row scans the compositions 32 pixels at a time.
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(256) pw_k_illum(PwParams P) {
    PW_ROUND_GUARD(P);
    const int gr = blockIdx.x * 8 + (int)threadIdx.x / 32, lane = threadIdx.x & 31;
    if (gr >= P.totalRows) return;
    const PawcsDev& S = P.streams[pw_stream_by_row(P, gr)];
    const StreamDev& D = S.sd;
    const int y = gr - D.rowBase;
    uint32_t carry = 0;  // outcome of the pixel before the chunk
    for (int x0 = 0; x0 < D.W; x0 += 32) {
        const int x = x0 + lane;
        const int p = y * D.W + x;
        const bool in = x < D.W && D.roi[p];
        uint32_t f = 0, m0 = 0, mL = 0;  // f: bit0 = outcome if the left neighbour made no update, bit1 = if it did
        if (in) {
            const uint32_t uvp = S.uv[p];
            m0 = S.illum[p] != 0;
            mL = D.roi[p] & 1u;  // the mask after the left neighbour's update
            const uint32_t u0 = uvp & 1u, u1 = (uvp >> 1) & 1u;
            f = (m0 ? u1 : u0) | ((mL ? u1 : u0) << 1);
        }
        // inclusive scan: F = f_lane o f_lane-1 o ... o f_x0
        uint32_t F = f;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, F, d);
            if (lane >= d) F = ((F >> (o & 1u)) & 1u) | (((F >> ((o >> 1) & 1u)) & 1u) << 1);
        }
        const uint32_t u = (F >> carry) & 1u;
        uint32_t prevU = __shfl_up_sync(0xffffffffu, u, 1);
        if (lane == 0) prevU = carry;
        if (x < D.W) S.uFinal[p] = in ? (uint8_t)(u | ((prevU ? mL : m0) ? 2u : 0u)) : (uint8_t)0;
        carry = __shfl_sync(0xffffffffu, u, 31);
    }
}

// ------------------------------------------------------------------------------------------
// global items: a BG pixel's dictionary event or an FG pixel's consultation. The first matching
// word in the pixel's sort table decides; only the replaceable word (last dictionary slot) changes
// features during a frame, so an item whose first non-replaceable match precedes the replaceable
// word is settled here, and the others go to the ordered scan. Run at the end of the pixel's local
// pass: it depends on nothing else that changes during the frame, so a pixel that does not rerun
// keeps its item.
// ------------------------------------------------------------------------------------------
__device__ void pw_item_pixel(const PawcsDev& S, int p, const PwRec& R, uint32_t col) {
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
    const PwThr th = pw_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    const uint32_t bits = R.bits;
    const uint8_t* lut = S.glut + (size_t)p * kPwGlutStride;
    int fixedPos = G, wrPos = G, fixedWord = -1;
    for (int g = 0; g < G; ++g) {
        const int w = lut[g];
        if (w == wr) {
            wrPos = g;
            continue;
        }
        if (fixedPos == G && pw_absdiff(pc->gw_color[w], col) <= th.color && pw_absdiff(bits, pc->gw_bits[w]) <= th.desc / 4u) {
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
// ordered compactions (raster order kept): mode 0 lists the critical global items, mode 1 the word
// weight contributions per word, mode 2 the pixels that update a neighbour. Blocks of kPwCompactBlk
// pixels: counts, offsets, scatter.
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ int pw_category(const PawcsDev& S, int p, int mode, int wr, uint32_t nrep) {
    if (!S.sd.roi[p]) return -1;
    const PwOut& O = S.out[p];
    if (mode == 0) return ((S.rec[p].flags & kRfItem) && (O.gflags & 4)) ? 0 : -1;
    if (mode == 2) return O.q != kPwNone ? 0 : -1;
    if (S.contrib[p] < 0.0f) return -1;
    // the replaceable word keeps only the contributions after its last replacement of the frame
    if (O.gword >= (uint32_t)S.G) return -1;
    if ((int)O.gword == wr && nrep > 0 && O.epoch != nrep) return -1;
    return (int)O.gword;
}

extern "C" __global__ void __launch_bounds__(256) pw_k_compact_count(PwParams P, int mode) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const int nb = (S.sd.npx + kPwCompactBlk - 1) / kPwCompactBlk;
    if ((int)blockIdx.x >= nb) return;
    __shared__ uint32_t cnt[kPwCats];
    if (threadIdx.x < kPwCats) cnt[threadIdx.x] = 0;
    __syncthreads();
    const int wr = S.pc->gdict[S.G - 1];
    const uint32_t nrep = S.pc->n_repl;
    for (int k = 0; k < kPwCompactBlk / 256; ++k) {
        const int p = blockIdx.x * kPwCompactBlk + k * 256 + threadIdx.x;
        if (p < S.sd.npx) {
            const int c = pw_category(S, p, mode, wr, nrep);
            if (c >= 0) atomicAdd(&cnt[c], 1u);
        }
    }
    __syncthreads();
    if (threadIdx.x < kPwCats) S.blkCounts[(size_t)blockIdx.x * kPwCats + threadIdx.x] = cnt[threadIdx.x];
}

// per category (one warp each): exclusive offsets over the blocks (in place), totals and the category
// bases of the word-major list; the compaction uses categories [0, ncat), the others are left empty
extern "C" __global__ void __launch_bounds__(1024) pw_k_compact_offsets(PwParams P, int ncat) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const int nb = (S.sd.npx + kPwCompactBlk - 1) / kPwCompactBlk;
    __shared__ uint32_t tot[kPwCats];
    const int lane = threadIdx.x & 31;
    for (int i = threadIdx.x; i < kPwCats; i += blockDim.x) tot[i] = 0;
    __syncthreads();
    for (int c = threadIdx.x >> 5; c < ncat; c += blockDim.x >> 5) {
        uint32_t run = 0;
        for (int b0 = 0; b0 < nb; b0 += 32) {
            const int b = b0 + lane;
            uint32_t* e = &S.blkCounts[(size_t)b * kPwCats + c];
            const uint32_t v = b < nb ? *e : 0u;
            uint32_t inc = v;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t o = __shfl_up_sync(0xffffffffu, inc, d);
                if (lane >= d) inc += o;
            }
            if (b < nb) *e = run + inc - v;
            run += __shfl_sync(0xffffffffu, inc, 31);
        }
        if (lane == 0) tot[c] = run;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t base = 0;
        for (int k = 0; k < kPwCats; ++k) {
            S.catInfo[k] = tot[k];
            S.catInfo[kPwCatBase + k] = base;
            base += tot[k];
        }
    }
}

extern "C" __global__ void __launch_bounds__(256) pw_k_compact_scatter(PwParams P, int mode) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const int nb = (D.npx + kPwCompactBlk - 1) / kPwCompactBlk;
    if ((int)blockIdx.x >= nb) return;
    __shared__ uint32_t warpCnt[8][kPwCats];
    __shared__ uint32_t run[kPwCats], passTot[kPwCats];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int wr = S.pc->gdict[S.G - 1];
    const uint32_t nrep = S.pc->n_repl;
    if (threadIdx.x < kPwCats)
        run[threadIdx.x] = S.catInfo[kPwCatBase + threadIdx.x] + S.blkCounts[(size_t)blockIdx.x * kPwCats + threadIdx.x];
    const float* fm = D.fm + (size_t)(D.ctl->frame_idx & 1ull) * kNumFloatMaps * D.npx;
    for (int k = 0; k < kPwCompactBlk / 256; ++k) {
        const int p = blockIdx.x * kPwCompactBlk + k * 256 + threadIdx.x;
        const int c = p < D.npx ? pw_category(S, p, mode, wr, nrep) : -1;
        uint32_t rank = 0;
        const int ncat = mode == 1 ? S.G : 1;
        for (int j = 0; j < ncat; ++j) {
            const unsigned m = __ballot_sync(0xffffffffu, c == j);
            if (c == j) rank = __popc(m & ((1u << lane) - 1u));
            if (lane == 0) warpCnt[w][j] = __popc(m);
        }
        __syncthreads();
        if (threadIdx.x < ncat) {
            // exclusive offsets of the warps within this pass, then the pass total
            uint32_t r = 0;
            for (int i = 0; i < 8; ++i) {
                const uint32_t v = warpCnt[i][threadIdx.x];
                warpCnt[i][threadIdx.x] = r;
                r += v;
            }
            passTot[threadIdx.x] = r;
        }
        __syncthreads();
        if (c >= 0) {
            const uint32_t pos = run[c] + warpCnt[w][c] + rank;
            if (mode == 0) {
                // two records per item (pixel, colour|bits, thresholds, descriptors 0-1; descriptor 2|event
                // flags, fixed position|word, and the global scan's speculative outcome)
                const PwRec& R = S.rec[p];
                const bool c3 = D.C == 3;
                const PwThr th = c3 ? pw3_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff)
                                    : pw_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
                const uint32_t g = S.gitem[p];
                const uint16_t* dt = S.descT + (size_t)p * (c3 ? 3 : 1);
                const uint32_t a = (c3 ? pw3_color(D.frame, p) : (uint32_t)D.frame[p]) | ((uint32_t)R.bits << 24);
                const uint32_t b = min(th.color, 65535u) | (min(th.desc / 4u, 65535u) << 16);
                const uint32_t d01 = c3 ? (uint32_t)dt[0] | ((uint32_t)dt[1] << 16) : (uint32_t)dt[0];
                const uint32_t d2 = c3 ? (uint32_t)dt[2] : 0u;
                S.itemList[2 * pos] = make_uint4((uint32_t)p, a, b, d01);
                S.itemList[2 * pos + 1] = make_uint4(d2 | ((uint32_t)(R.flags & (kRfEvent | kRfRepDraw)) << 16),
                                                     ((g >> 6) & 63u) | ((g & 63u) << 8), 0u, 0u);
            } else if (mode == 2) {
                S.updList[pos] = (uint32_t)p;
            } else {
                S.contribList[pos] = S.contrib[p];
            }
        }
        __syncthreads();
        if (threadIdx.x < ncat) run[threadIdx.x] += passTot[threadIdx.x];
        __syncthreads();
    }
}

// per 2x2 cell of the spatial maps: the cell's (at most four) items in raster order (:786-791,
// :805-812); final = 1 also writes the frame's map values and word contributions
extern "C" __global__ void pw_k_cells(PwParams P, int final) {
    PW_ROUND_GUARD(P);
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.totalCells) return;
    int si = 0;
    while (si + 1 < P.nStreams && c >= P.streams[si].gwW * P.streams[si].gwH) {
        c -= P.streams[si].gwW * P.streams[si].gwH;
        ++si;
    }
    const PawcsDev& S = P.streams[si];
    const StreamDev& D = S.sd;
    const PawcsCtl* pc = S.pc;
    const int cx = c % S.gwW, cy = c / S.gwW;
    const size_t ncell = (size_t)S.gwW * S.gwH;
    const int G = S.G;
    const int wr = pc->gdict[G - 1];
    int ws[4];
    float vs[4];
    int nw = 0;
    uint32_t wrE = 0;
    float wrV = S.gmap[(size_t)wr * ncell + c];
    int wrTouched = 0;
    for (int k = 0; k < 4; ++k) {
        const int x = 2 * cx + (k & 1), y = 2 * cy + (k >> 1);
        if (x >= D.W || y >= D.H) continue;
        const int p = y * D.W + x;
        if (!D.roi[p]) continue;
        const PwRec& R = S.rec[p];
        if (!(R.flags & kRfItem)) {
            if (final) S.contrib[p] = -1.0f;
            continue;
        }
        PwOut& O = S.out[p];
        const uint32_t w = O.gword;
        float contrib = -1.0f;
        if (w == kPwNone) {
            if (!(R.flags & kRfBG)) O.segm = 255;
        } else {
            float* v;
            if ((int)w == wr) {
                if (O.epoch != wrE) {
                    wrV = 0.0f;  // the word was replaced (its map zeroed) since the cell's last look
                    wrE = O.epoch;
                }
                v = &wrV;
                wrTouched = 1;
            } else {
                int j = 0;
                while (j < nw && ws[j] != (int)w) ++j;
                if (j == nw) {
                    ws[nw] = (int)w;
                    vs[nw] = S.gmap[(size_t)w * ncell + c];
                    ++nw;
                }
                v = &vs[j];
            }
            if (R.flags & kRfBG) {
                if (*v < R.sumW) {
                    *v = *v + R.sumW;
                    contrib = R.sumW;
                }
            } else {
                const float div = (R.flags & kRfFlat) ? 2.0f : 4.0f;
                O.segm = (R.sumW + *v / div < R.thrW) ? 255 : 0;
            }
        }
        if (final) S.contrib[p] = contrib;
    }
    if (!final) return;
    for (int j = 0; j < nw; ++j) S.gmap[(size_t)ws[j] * ncell + c] = vs[j];
    // the replaceable word: values after the frame's last replacement; zero elsewhere when replaced
    const uint32_t nrep = pc->n_repl;
    if (nrep == 0) {
        if (wrTouched) S.gmap[(size_t)wr * ncell + c] = wrV;
    } else {
        S.gmap[(size_t)wr * ncell + c] = (wrTouched && wrE == nrep) ? wrV : 0.0f;
    }
}

// neighbour-update gate and target (:839-848): the draws before it depend on the global outcome
extern "C" __global__ void __launch_bounds__(256) pw_k_nbr(PwParams P) {
    PW_ROUND_GUARD(P);
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
    if (x >= D.W || y >= D.H) return;
    const int p = y * D.W + x;
    if (!D.roi[p]) return;
    const PwRec& R = S.rec[p];
    PwOut& O = S.out[p];
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    uint32_t k = R.kScan;
    uint8_t segm;
    if (R.flags & kRfBG) {
        segm = 0;
        ++k;  // the event draw (:774), taken whatever its outcome
        if (R.flags & kRfEvent) {
            const bool noMatch = O.gword == kPwNone || (O.gflags & 1);
            if (noMatch) ++k;  // the replacement draw (:785), taken when no word matched
        }
    } else {
        if (!(R.flags & kRfFlat)) ++k;  // the consultation gate draw
        if (!(R.flags & kRfItem)) O.segm = 255;
        segm = O.segm;
    }
    if (R.flags & kRfBG) O.segm = 0;
    const int border = (R.flags & kRfBorder) != 0, flat = (R.flags & kRfFlat) != 0;
    const int moving = S.pc->moving_cam;
    bool upd = false;
    if (!segm) upd = pw_mod(pw_draw(D.seed, t, (uint32_t)p, k++), R.rate) == 0u;
    upd = upd || border || moving;
    // the previous round's loop inputs (round 0: no update known to the targets' local passes)
    const uint32_t oldQ = P.round == 0 ? kPwNone : O.q;
    const uint16_t oldK = O.kLoop;
    const float oldThr = O.thrW;
    O.q = kPwNone;
    if (upd) {
        const uint32_t r = pw_draw(D.seed, t, (uint32_t)p, k++);
        int nx, ny;
        if (flat || border || moving) {
            const int i = (int)(r % 24u);
            nx = x + pw_nb5[i][0];
            ny = y + pw_nb5[i][1];
        } else {
            const int i = (int)(r % 8u);
            nx = x + pw_nb3[i][0];
            ny = y + pw_nb3[i][1];
        }
        nx = nx < 2 ? 2 : nx >= D.W - 2 ? D.W - 3 : nx;
        ny = ny < 2 ? 2 : ny >= D.H - 2 ? D.H - 3 : ny;
        const int q = ny * D.W + nx;
        if (D.roi[q]) O.q = (uint32_t)q;
    }
    O.kLoop = (uint16_t)k;
    O.thrW = R.thrW;
    O.qPrev = oldQ;
    O.chg = (uint8_t)(O.q != oldQ || (O.q != kPwNone && (O.kLoop != oldK || O.thrW != oldThr)));
}

// the neighbour-update loop of updater p on target q (:847-880; one channel: the reference updates a
// copy of each word, so only the weight sum and the draws count). p sees q's dictionary before q's own
// scan (p < q: frame-start words, the last one replaced by the earlier updater rs, if any) or after it
// (p >= q: the scanned words with their illumination marks). Returns the weight sum; k advances by
// the loop's draws; reachedLast tells whether the loop looked at the last word (the only one rs changes).
__device__ float pw_nbr_loop(const PawcsDev& S, uint32_t t, int cur, int nxt, int boot, unsigned long long off, int p,
                             int q, uint32_t rs, uint32_t& k, bool& reachedLast) {
    const StreamDev& D = S.sd;
    const float* fm = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
    const PwRec& R = S.rec[p];
    const uint32_t col = D.frame[p], desc = S.descT[p];
    const PwThr th = pw_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    const int flat = (R.flags & kRfFlat) != 0;
    PwWordSrc ws;
    ws.S = &S;
    ws.q = q;
    ws.L = S.L;
    ws.t = t;
    ws.qcol = D.frame[q];
    ws.qdesc = S.descT[q];
    uint8_t segmQ;
    uint32_t lastDescQ;
    if (p < q) {
        ws.buf = cur;
        ws.m = 0;
        segmQ = 0;
        lastDescQ = D.lastDesc[q];
    } else {
        const PwRec& Rq = S.rec[q];
        ws.buf = nxt;
        ws.m = (S.uFinal[q] & 2) ? Rq.m1 : Rq.m0;
        segmQ = S.out[q].segm;
        // the pixel's last descriptor is updated at the end of its own processing (:925-926)
        lastDescQ = p == q ? D.lastDesc[q] : S.descT[q];
    }
    ws.repl = rs != kPwNone;
    if (ws.repl) {
        ws.rcol = D.frame[rs];
        ws.rdesc = S.descT[rs];
        ws.rincr = S.rec[rs].incr;
    }
    float nsum = 0.0f;
    reachedLast = false;
    for (int j = 0; j < S.L && nsum < R.thrW; ++j) {
        if (j == S.L - 1) reachedLast = true;
        uint32_t c, d, o, f, l;
        pw_word(ws, j, c, d, o, f, l);
        const uint32_t cd = pw_absdiff(col, c);
        if (cd <= th.color && (uint32_t)__popc(desc ^ d) <= th.desc) {
            nsum += pw_weight(o, f, l, t, off);
        } else if (!segmQ && flat && (boot || pw_mod(pw_draw(D.seed, t, (uint32_t)p, k++), R.rate) == 0u)) {
            if (cd <= th.color && (uint32_t)__popc(desc ^ lastDescQ) <= th.desc / 2u) nsum += pw_weight(o, f, l, t, off);
        }
    }
    return nsum;
}

// neighbour updates, pass 1: every updater's loop (one thread each, over the compacted list), as if no
// earlier updater of its target had replaced the target's last word
extern "C" __global__ void __launch_bounds__(256) pw_k_nbr_loops(PwParams P) {
    PW_ROUND_GUARD(P);
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const uint32_t n = S.catInfo[0];
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    const int cur = (int)(D.ctl->frame_idx & 1ull), nxt = cur ^ 1;
    const int boot = t <= (uint32_t)kBootWin;
    const unsigned long long off = S.pc->lword_offset;
    const float initW = 1.0f / (float)off;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int p = (int)S.updList[i];
        PwOut& O = S.out[p];
        uint32_t k = O.kLoop;
        bool reachedLast;
        const float nsum = pw_nbr_loop(S, t, cur, nxt, boot, off, p, (int)O.q, kPwNone, k, reachedLast);
        O.kEnd = (uint16_t)k;
        O.rflags = (uint8_t)((nsum < initW ? 1 : 0) | (reachedLast ? 2 : 0));
    }
}

// neighbour updates, pass 2 (per target, raster order over its <= 25 updaters): the latest updater of
// each group that replaces the last word is the replacement source the next ones see; a later updater
// whose loop reached that word is redone with it (the earlier words are the same either way)
extern "C" __global__ void __launch_bounds__(256) pw_k_replace(PwParams P) {
    PW_ROUND_GUARD(P);
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int qx = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int qy = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
    if (qx >= D.W || qy >= D.H) return;
    const int q = qy * D.W + qx;
    if (!D.roi[q]) return;
    const StreamCtl* ctl = D.ctl;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int cur = (int)(ctl->frame_idx & 1ull), nxt = cur ^ 1;
    const int boot = t <= (uint32_t)kBootWin;
    const unsigned long long off = S.pc->lword_offset;
    const float initW = 1.0f / (float)off;
    uint32_t before = kPwNone, after = kPwNone;
    for (int dy = -2; dy <= 2; ++dy)
        for (int dx = -2; dx <= 2; ++dx) {
            const int px = qx + dx, py = qy + dy;
            if (px < 0 || py < 0 || px >= D.W || py >= D.H) continue;
            const int p = py * D.W + px;
            if (!D.roi[p]) continue;
            // p == q happens when the clamped neighbour position falls back onto the pixel itself (at
            // the ROI's outer rows and columns): the update then follows the pixel's own processing
            PwOut& O = S.out[p];
            if (O.q != (uint32_t)q) continue;
            const uint32_t rs = p < q ? before : after;
            uint8_t rf = O.rflags;
            if (rs != kPwNone && (rf & 2)) {
                uint32_t k = O.kLoop;
                bool reachedLast;
                const float nsum = pw_nbr_loop(S, t, cur, nxt, boot, off, p, q, rs, k, reachedLast);
                rf = (uint8_t)((nsum < initW ? 1 : 0) | (reachedLast ? 2 : 0));
                O.kEnd = (uint16_t)k;
                O.rflags = rf;
            }
            if (rf & 1) {
                if (p < q) before = (uint32_t)p;
                else after = (uint32_t)p;
            }
        }
    S.repBefore[q] = before;
    S.repAfter[q] = after;
}

// pixels whose replacement source changed since their local pass are redone next round
extern "C" __global__ void __launch_bounds__(256) pw_k_dirty(PwParams P) {
    PW_ROUND_GUARD(P);
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
    bool dirty = false;
    if (x < D.W && y < D.H) {
        const int p = y * D.W + x;
        dirty = D.roi[p] && S.repBefore[p] != S.rec[p].rsrc;
    }
    const unsigned b = __ballot_sync(0xffffffffu, dirty);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&P.flags[0], (unsigned)__popc(b));
}

// end of a fixed-point round (one thread): no dirty pixel means the fixed point is reached; the
// round count is recorded and the flag makes the rounds enqueued after this one return at once
extern "C" __global__ void pw_k_round_end(PwParams P) {
    PW_ROUND_GUARD(P);
    if (P.flags[0] == 0u) {
        P.flags[4] = (unsigned)P.round + 1u;
        __threadfence();
        P.flags[3] = 1u;
    }
}

// ------------------------------------------------------------------------------------------
// commit of the frame's pixel loop: final dictionaries (illumination updates, later neighbour
// replacements), feedback maps (:764-771, :800-806, :895-914), illumination mask, last colour and
// descriptor, raw mask (as the post-processing "intent" word) and draw counters
// ------------------------------------------------------------------------------------------
extern "C" __global__ void __launch_bounds__(256) pw_k_commit(PwParams P) {
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
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
        const uint32_t col = D.frame[p], desc = S.descT[p];
        flat = (R.flags & kRfFlat) != 0;
        // dictionary: illumination updates, then a later neighbour's replacement of the last slot
        const uint8_t u = S.uFinal[p];
        const uint32_t m = (u & 2) ? R.m1 : R.m0;
        for (int s = 0; s < S.L; ++s)
            if (m & (1u << s)) {
                const size_t a = pw_slot(S, nxt, s, p);
                S.wColor[a] = (uint8_t)col;
                S.wDesc[a] = (uint16_t)desc;
            }
        const uint32_t ra = S.repAfter[p];
        if (ra != kPwNone) {
            const size_t a = pw_slot(S, nxt, S.L - 1, p);
            S.wColor[a] = D.frame[ra];
            S.wDesc[a] = S.descT[ra];
            S.wOcc[a] = S.rec[ra].incr;
            S.wFirst[a] = t;
            S.wLast[a] = t;
        }
        // illumination mask at the end of the frame (:686-690, :889-890): the right neighbour's
        // update sets 1 & ROI; else the own update leaves 2-1 = 1; else the start value (1 & ROI
        // after the left neighbour's update) minus one
        const int roiBit = D.roi[p] & 1;
        const int uRight = (x + 1 < D.W && D.roi[p + 1]) ? (S.uFinal[p + 1] & 1) : 0;
        const int mStart = (x > 0 && D.roi[p - 1] && (S.uFinal[p - 1] & 1)) ? roiBit : (int)S.illum[p];
        int mEnd;
        if (uRight) mEnd = roiBit;
        else if (u & 1) mEnd = 1;
        else mEnd = mStart > 0 ? mStart - 1 : 0;
        S.illum[p] = (uint8_t)mEnd;
        // feedback
        float fLT, fST;
        pw_factors(t, (int)S.nmv, &fLT, &fST);
        const float* fc = D.fm + (size_t)cur * kNumFloatMaps * D.npx;
        float* fn = D.fm + (size_t)nxt * kNumFloatMaps * D.npx;
        const int npx = D.npx;
        float dLT = fc[FM_DMIN_LT * npx + p], dST = fc[FM_DMIN_ST * npx + p];
        float rLT = fc[FM_RAW_LT * npx + p], rST = fc[FM_RAW_ST * npx + p];
        const float nmc = (float)R.minColor / 255.0f, nmd = (float)R.minDesc / 16.0f;
        const float nd0 = (nmc < nmd) ? nmd : nmc;  // std::max
        if (R.flags & kRfBG) {
            dLT = dLT * (1.0f - fLT) + nd0 * fLT;
            dST = dST * (1.0f - fST) + nd0 * fST;
            rLT = rLT * (1.0f - fLT);
            rST = rST * (1.0f - fST);
        } else {
            const float q = (R.thrW - R.sumW) / R.thrW;
            const float nd = (nd0 < q) ? q : nd0;
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
        // R < std::pow(1+2*dmin, 2) in double: exact via the split x*x = hi + lo
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
        D.lastCol[p] = (uint8_t)col;
        D.lastDesc[p] = (uint16_t)desc;
        D.intent[p] = O.segm ? (kInValid | kInFG) : kInValid;
        D.kctr[p] = O.q != kPwNone ? O.kEnd : O.kLoop;  // the draw count after the pixel's updates
    } else if (in) {
        D.intent[p] = 0u;
    }
    const unsigned b = __ballot_sync(0xffffffffu, act && flat);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(&S.pc->nflat_acc, (unsigned long long)__popc(b));
}

// global word weights (:789-790): ordered float sums of the frame's contributions, one block per
// (stream, word) over the word's compacted list; the replaceable word restarts from zero at the
// frame's last replacement (its list holds only the contributions after it)
extern "C" __global__ void __launch_bounds__(256) pw_k_weights(PwParams P) {
    const int si = blockIdx.x / kPwMaxGlobal, w = blockIdx.x % kPwMaxGlobal;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    if (w >= S.G) return;
    PawcsCtl* pc = S.pc;
    const int wr = pc->gdict[S.G - 1];
    const uint32_t nrep = pc->n_repl;
    const bool isWr = w == wr;
    const uint32_t n = S.catInfo[w], base = S.catInfo[kPwCatBase + w];
    __shared__ float buf[1024];
    float acc = (isWr && nrep > 0) ? 0.0f : pc->gw_weight[w];
    for (uint32_t c0 = 0; c0 < n; c0 += 1024) {
        const uint32_t cnt = min(1024u, n - c0);
        for (uint32_t i = threadIdx.x; i < cnt; i += blockDim.x) buf[i] = S.contribList[base + c0 + i];
        __syncthreads();
        if (threadIdx.x == 0)
            for (uint32_t i = 0; i < cnt; ++i) acc = acc + buf[i];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        pc->gw_weight[w] = acc;
        if (isWr && nrep > 0) {
            pc->gw_color[w] = pc->wr_color;
            pc->gw_desc[w] = pc->wr_desc;
            pc->gw_desc2[w] = pc->wr_desc2;
            pc->gw_bits[w] = pc->wr_bits;
        }
    }
}

// ------------------------------------------------------------------------------------------
// end-of-frame global words (:1300-1334)
// ------------------------------------------------------------------------------------------
// per word: every 256/512 frames the weight becomes the map sum (double, raster order); every
// 8/16 frames the map decays where the previous dilated mask was background, then a 3x3 blur
__device__ __forceinline__ void pw_gw_rates(uint32_t t, int* recalc, int* update) {
    const uint32_t rate = t <= (uint32_t)kBootWin ? 8u : 16u;
    *recalc = (t % (rate << 5)) == 0u;
    *update = (t % rate) == 0u;
}

extern "C" __global__ void pw_k_gw_recalc(PwParams P) {
    const int si = blockIdx.x / kPwMaxGlobal, w = blockIdx.x % kPwMaxGlobal;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    if (w >= S.G) return;
    PawcsCtl* pc = S.pc;
    int recalc, update;
    pw_gw_rates((uint32_t)(S.sd.ctl->frame_idx + 1ull), &recalc, &update);
    if (!recalc || !(pc->gw_weight[w] > 0.0f)) return;
    const size_t n = (size_t)S.gwW * S.gwH;
    float* m = S.gmap + (size_t)w * n;
    __shared__ float wsum;
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (size_t i = 0; i < n; ++i) s += (double)m[i];
        wsum = (float)s;
        pc->gw_weight[w] = wsum < 1.0f ? 0.0f : wsum;
    }
    __syncthreads();
    if (wsum < 1.0f)
        for (size_t i = threadIdx.x; i < n; i += blockDim.x) m[i] = 0.0f;
}

// decay (accumulateProduct with the INTER_NEAREST down-scaled previous inverted dilated mask) and the
// first half of the blur (row sums, double); one block row per map row
extern "C" __global__ void pw_k_gw_decay(PwParams P, double* rowsum) {
    const int si = blockIdx.y / kPwMaxGlobal, w = blockIdx.y % kPwMaxGlobal;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    if (w >= S.G) return;
    int recalc, update;
    pw_gw_rates((uint32_t)(S.sd.ctl->frame_idx + 1ull), &recalc, &update);
    if (!update || !(S.pc->gw_weight[w] > 0.0f)) return;
    const int gw = S.gwW, gh = S.gwH, W = S.sd.W, H = S.sd.H;
    const size_t n = (size_t)gw * gh;
    float* m = S.gmap + (size_t)w * n;
    double* rs = rowsum + ((size_t)si * kPwMaxGlobal + w) * n;
    const double ifx = 1.0 / ((double)gw / W), ify = 1.0 / ((double)gh / H);
    for (int yy = blockIdx.x; yy < gh; yy += gridDim.x) {
        int sy = (int)floor(yy * ify);
        sy = sy < H - 1 ? sy : H - 1;
        for (int xx = threadIdx.x; xx < gw; xx += blockDim.x) {
            int sx = (int)floor(xx * ifx);
            sx = sx < W - 1 ? sx : W - 1;
            const size_t i = (size_t)yy * gw + xx;
            if (S.sd.dilInv[(size_t)sy * W + sx]) {
                const float prod = m[i] * -0.1f;
                m[i] = m[i] + prod;
            }
        }
        __syncthreads();
        for (int xx = threadIdx.x; xx < gw; xx += blockDim.x) {
            const int x0 = xx > 0 ? xx - 1 : 0, x1 = xx < gw - 1 ? xx + 1 : gw - 1;
            const size_t r = (size_t)yy * gw;
            rs[r + xx] = ((double)m[r + x0] + (double)m[r + xx]) + (double)m[r + x1];
        }
    }
}

// second half of the blur (column sums * 1/9, to float), the weight decay and, in the last block,
// the one-pass dictionary sort by weight
extern "C" __global__ void pw_k_gw_blur(PwParams P, const double* rowsum) {
    const int si = blockIdx.y / kPwMaxGlobal, w = blockIdx.y % kPwMaxGlobal;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    if (w >= S.G) return;
    int recalc, update;
    pw_gw_rates((uint32_t)(S.sd.ctl->frame_idx + 1ull), &recalc, &update);
    if (!update || !(S.pc->gw_weight[w] > 0.0f)) return;
    const int gw = S.gwW, gh = S.gwH;
    const size_t n = (size_t)gw * gh;
    float* m = S.gmap + (size_t)w * n;
    const double* rs = rowsum + ((size_t)si * kPwMaxGlobal + w) * n;
    for (int yy = blockIdx.x; yy < gh; yy += gridDim.x) {
        const int y0 = yy > 0 ? yy - 1 : 0, y1 = yy < gh - 1 ? yy + 1 : gh - 1;
        for (int xx = threadIdx.x; xx < gw; xx += blockDim.x) {
            const double tsum = (rs[(size_t)y0 * gw + xx] + rs[(size_t)yy * gw + xx]) + rs[(size_t)y1 * gw + xx];
            m[(size_t)yy * gw + xx] = (float)(tsum * (1.0 / 9.0));
        }
    }
}

// weight decay and the dictionary's bubble step (after all maps are final)
extern "C" __global__ void pw_k_gw_sort(PwParams P) {
    const int si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    PawcsCtl* pc = S.pc;
    int recalc, update;
    pw_gw_rates((uint32_t)(S.sd.ctl->frame_idx + 1ull), &recalc, &update);
    for (int g = 0; g < S.G; ++g) {
        const int w = pc->gdict[g];
        if (update && pc->gw_weight[w] > 0.0f) pc->gw_weight[w] *= 0.9f;
        if (g > 0 && pc->gw_weight[pc->gdict[g]] > pc->gw_weight[pc->gdict[g - 1]]) {
            const int tmp = pc->gdict[g];
            pc->gdict[g] = pc->gdict[g - 1];
            pc->gdict[g - 1] = tmp;
        }
    }
}

// per-pixel global word order: one bubble pass on the local map weights (:1318-1330, :415-427);
// mode 0: only on update frames (apply), 1: always (refreshModel), 2: when an automatic reset is pending
extern "C" __global__ void __launch_bounds__(256) pw_k_lut_sort(PwParams P, int mode) {
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    if (mode == 0) {
        int recalc, update;
        pw_gw_rates((uint32_t)(D.ctl->frame_idx + 1ull), &recalc, &update);
        if (!update) return;
    } else if (mode == 2 && S.pc->reset_pending == 0) {
        return;
    }
    const int lt = t0 - D.tileBase;
    const int x = (lt % D.tilesX) * kTileW + (int)threadIdx.x % kTileW;
    const int y = (lt / D.tilesX) * kTileH + (int)threadIdx.x / kTileW;
    if (x >= D.W || y >= D.H) return;
    const int p = y * D.W + x;
    if (!D.roi[p]) return;
    const size_t n = (size_t)S.gwW * S.gwH;
    const size_t cidx = (size_t)(y / 2) * S.gwW + (x / 2);
    uint8_t* lut = S.glut + (size_t)p * kPwGlutStride;
    uint8_t o[kPwMaxGlobal];
    for (int g = 0; g < S.G; ++g) o[g] = lut[g];
    float last = S.gmap[(size_t)o[0] * n + cidx];
    for (int g = 1; g < S.G; ++g) {
        const float c = S.gmap[(size_t)o[g] * n + cidx];
        if (c > last) {
            const uint8_t tmp = o[g];
            o[g] = o[g - 1];
            o[g - 1] = tmp;
        } else {
            last = c;
        }
    }
    for (int g = 0; g < S.G; ++g) lut[g] = o[g];
}

// blinks (:1443-1446) and the 3x3 closing of the raw mask (:1447)
extern "C" __global__ void __launch_bounds__(256) pw_k_blink_close(PwParams P) {
    const int t0 = blockIdx.x;
    if (t0 >= P.totalTiles) return;
    const PawcsDev& S = P.streams[pw_stream_by_tile(P, t0)];
    const StreamDev& D = S.sd;
    const int lt = t0 - D.tileBase;
    const int x0 = (lt % D.tilesX) * kTileW, y0 = (lt / D.tilesX) * kTileH;
    constexpr int IW = kTileW + 4, IH = kTileH + 4, DW = kTileW + 2, DH = kTileH + 2;
    __shared__ uint8_t raw[IW * IH];
    __shared__ uint8_t dil[DW * DH];
    const int W = D.W, H = D.H;
    for (int i = threadIdx.x; i < IW * IH; i += blockDim.x) {
        const int gy = y0 - 2 + i / IW, gx = x0 - 2 + i % IW;
        raw[i] = (gy >= 0 && gy < H && gx >= 0 && gx < W && (D.intent[gy * W + gx] & kInFG)) ? 255 : 0;
    }
    __syncthreads();
    // dilation over the clipped 3x3 window (out-of-image pixels never win)
    for (int i = threadIdx.x; i < DW * DH; i += blockDim.x) {
        const int ry = i / DW, rx = i % DW;
        uint8_t v = 0;
        for (int dy = 0; dy < 3; ++dy)
            for (int dx = 0; dx < 3; ++dx) v |= raw[(ry + dy) * IW + rx + dx];
        dil[i] = v;
    }
    __syncthreads();
    const int lx = threadIdx.x % kTileW, ly = threadIdx.x / kTileW;
    const int x = x0 + lx, y = y0 + ly;
    bool rawBit = false, closedBit = false;
    if (x < W && y < H) {
        const int q = y * W + x;
        const uint8_t r = raw[(ly + 2) * IW + lx + 2];
        const uint8_t cb = r ^ D.lastRawFG[q];
        D.blinks[q] = cb | D.lastRawBlink[q];
        D.lastRawBlink[q] = cb;
        D.lastRawFG[q] = r;
        // erosion of the dilated mask over the clipped window
        uint8_t v = 255;
        for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
                const int gx = x + dx, gy = y + dy;
                if (gx < 0 || gx >= W || gy < 0 || gy >= H) continue;
                v &= dil[(ly + 1 + dy) * DW + lx + 1 + dx];
            }
        rawBit = r != 0;
        closedBit = v != 0;
    }
    // each warp is one 32-pixel tile row: its ballots are the row's words of the raw and closed masks
    const unsigned rawW = __ballot_sync(0xffffffffu, rawBit), closedW = __ballot_sync(0xffffffffu, closedBit);
    if (lx == 0 && y < H) {
        const size_t o = (size_t)y * D.rowWords + x0 / 32;
        bit_plane(D, BP_RAW)[o] = rawW;
        bit_plane(D, BP_CLOSED)[o] = closedW;
    }
}

// down-sampled frame (INTER_AREA, integral scale), its rolling averages (accumulateWeighted) and the
// per-pixel |LT - ST| of the motion analysis (:1475-1478); one thread per down-sampled pixel
extern "C" __global__ void pw_k_ds(PwParams P) {
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const int nds = D.dsW * D.dsH;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nds) return;
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    float fLT, fST;
    pw_factors(t, (int)S.nmv, &fLT, &fST);
    const int bx = i % D.dsW, by = i / D.dsW;
    const uint8_t* fr = D.frame;
    const int W = D.W;
    const uint8_t vb = area_resample(D.W, D.H, D.dsW, D.dsH, bx, by,
                                     [&](int sx, int sy) { return (int)fr[(size_t)sy * W + sx]; });
    const float lt = (float)vb * fLT + D.dsLT[i] * (1.0f - fLT);
    const float st = (float)vb * fST + D.dsST[i] * (1.0f - fST);
    D.dsLT[i] = lt;
    D.dsST[i] = st;
    S.dsFrame[i] = vb;
    S.dsAbs[i] = S.dsRoi[i] ? fabsf(lt - st) : 0.0f;
}

// ------------------------------------------------------------------------------------------
// frame level (:1462-1516): LBSP threshold LUT, camera-motion analysis, automatic model reset
// decision; one block per stream
// ------------------------------------------------------------------------------------------
extern "C" __global__ void pw_k_epilogue(PwParams P) {
    const int si = blockIdx.x;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    const StreamDev& D = S.sd;
    StreamCtl* ctl = D.ctl;
    PawcsCtl* pc = S.pc;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int boot = t <= (uint32_t)kBootWin;
    float fLT, fST;
    pw_factors(t, (int)S.nmv, &fLT, &fST);
    (void)fST;
    const int nds = D.dsW * D.dsH;
    // ordered float sum of |LT - ST| over the down-sampled ROI (lv::L1dist, math.hpp:255-268): the
    // block stages the terms in shared memory, one thread adds them in order
    __shared__ float terms[2048];
    float l1 = 0.0f;
    for (int c0 = 0; c0 < nds; c0 += 2048) {
        const int cnt = min(2048, nds - c0);
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) terms[i] = S.dsAbs[c0 + i];
        __syncthreads();
        if (threadIdx.x == 0)
            for (int i = 0; i < cnt; ++i) l1 = l1 + terms[i];
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const float ratio = l1 / (float)pc->ds_roi_count;
    pc->frame_ratio = ratio;
    // LBSP threshold LUT (:1462-1473)
    const float nonflat = (float)(ctl->n_rel - pc->nflat_acc) / (float)ctl->n_rel;
    const float rel = S.relThr;
    const float offs = (float)S.lbspOff;
    if (nonflat < 0.1f && pc->last_nonflat_ratio < 0.1f) {
        for (int k = 0; k <= 255; ++k) {
            const float v = (offs + (float)k * rel) / 4;
            const int r = __float2int_rn(v);
            const int lim = r < 0 ? 0 : r > 255 ? 255 : r;
            if ((int)ctl->lut[k] > lim) --ctl->lut[k];
        }
    } else if (nonflat > 0.5f && pc->last_nonflat_ratio > 0.5f) {
        const float v = offs + 255 * rel;
        const int r = __float2int_rn(v);
        const int lim = r < 0 ? 0 : r > 255 ? 255 : r;
        for (int k = 0; k <= 255; ++k)
            if ((int)ctl->lut[k] < lim) ++ctl->lut[k];
    }
    pc->last_nonflat_ratio = nonflat;
    pc->nflat_acc = 0;
    pc->reset_pending = 0;
    // automatic model reset (:1479-1513): the block is entered when the reset is enabled or the camera
    // moves; the camera-motion comparison of frames 500, 1000, ... (pw_k_motion_*) and the reset decision
    // (pw_k_reset_decide) follow
    if (!ctl->auto_reset && ratio >= 45.0f * 2) ctl->auto_reset = 1;
    pc->reset_block = ctl->auto_reset || pc->moving_cam;
}

// reset decision of the frame-level block (:1509-1513)
extern "C" __global__ void pw_k_reset_decide(PwParams P) {
    const int si = blockIdx.x;
    if (si >= P.nStreams || threadIdx.x != 0) return;
    const PawcsDev& S = P.streams[si];
    StreamCtl* ctl = S.sd.ctl;
    PawcsCtl* pc = S.pc;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    const int boot = t <= (uint32_t)kBootWin;
    const float ratio = pc->frame_ratio;
    if (pc->reset_block) {
        if (ctl->frames_since_reset > (unsigned long long)kBootWin * 2) {
            ctl->auto_reset = 0;
        } else if (ratio >= 45.0f && ctl->cooldown == 0) {
            ctl->frames_since_reset = 0;
            pc->reset_pending = 1;
        } else if (!boot) {
            ++ctl->frames_since_reset;
        }
    }
}

// closes the frame: frame index, cooldown, factors of the next frame's final-segmentation averages
extern "C" __global__ void pw_k_close(PwParams P) {
    const int si = blockIdx.x * blockDim.x + threadIdx.x;
    if (si >= P.nStreams) return;
    const PawcsDev& S = P.streams[si];
    StreamCtl* ctl = S.sd.ctl;
    PawcsCtl* pc = S.pc;
    const uint32_t t = (uint32_t)(ctl->frame_idx + 1ull);
    if (pc->reset_pending == 1) {
        float fLT, fST;
        pw_factors(t, (int)S.nmv, &fLT, &fST);
        const int boot = t <= (uint32_t)kBootWin;
        const unsigned long long nlt = boot ? (unsigned long long)(S.nmv / 2) : (unsigned long long)S.nmv;
        ctl->cooldown = nlt / 4;
    }
    if (ctl->cooldown > 0) --ctl->cooldown;
    ctl->frame_idx = t;
    // factors of the next frame (used by the median kernel's final-segmentation averages)
    float fLT, fST;
    pw_factors((unsigned long long)t + 1ull, (int)S.nmv, &fLT, &fST);
    ctl->fLT = fLT;
    ctl->fST = fST;
    ctl->bLT = (float)((1.0 / 255) * (double)fLT);
    ctl->bST = (float)((1.0 / 255) * (double)fST);
}

// ------------------------------------------------------------------------------------------
// refreshModel (:107-429), one channel
// ------------------------------------------------------------------------------------------
// local resampling: 98 draws from the 7x7 neighbourhood per pixel, then (initialization) the
// random fill of empty slots; one thread per pixel
extern "C" __global__ void __launch_bounds__(128) pw_k_refresh_local(PawcsDev S, uint32_t t, int buf, int baseOcc,
                                                                      float decr, int force, int onlyPending,
                                                                      int useDil) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    const StreamDev& D = S.sd;
    if (p >= D.npx) return;
    if (onlyPending && S.pc->reset_pending == 0) return;
    if (!D.roi[p]) return;
    // m_oLastFGMask_dilated: the complement of the stored inverted mask (all clear at initialization)
    if (!(force || !useDil || D.dilInv[p] != 0)) return;
    const int L = S.L;
    const int x0 = p % D.W, y0 = p / D.W;
    const unsigned long long off = S.pc->lword_offset;
    const float* fm = D.fm + (size_t)buf * kNumFloatMaps * D.npx;
    const PwThr th = pw_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
    uint8_t wc[kPwMaxLocal];
    uint16_t wd[kPwMaxLocal];
    uint32_t wo[kPwMaxLocal], wf[kPwMaxLocal], wl[kPwMaxLocal];
    for (int j = 0; j < L; ++j) {
        const size_t a = pw_slot(S, buf, j, p);
        wc[j] = S.wColor[a];
        wd[j] = S.wDesc[a];
        wo[j] = S.wOcc[a];
        wf[j] = S.wFirst[a];
        wl[j] = S.wLast[a];
    }
    // empty slots carry first == kPwNone (initialization only)
    if (decr > 0.0f)
        for (int j = 0; j < L; ++j)
            if (wf[j] != kPwNone) wo[j] -= (uint32_t)(decr * (float)wo[j]);
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
        const uint32_t scol = D.lastCol[sp], sdesc = D.lastDesc[sp];
        int i;
        for (i = 0; i < L; ++i) {
            if (wf[i] == kPwNone) continue;
            if (pw_absdiff(scol, wc[i]) <= th.color && (uint32_t)__popc(sdesc ^ wd[i]) <= th.desc) {
                wo[i] += 1;
                wl[i] = t;
                break;
            }
        }
        if (i == L) {
            i = L - 1;
            wc[i] = (uint8_t)scol;
            wd[i] = (uint16_t)sdesc;
            wo[i] = (uint32_t)baseOcc;
            wf[i] = t;
            wl[i] = t;
        }
        while (i > 0 && (wf[i - 1] == kPwNone ||
                         pw_weight(wo[i], wf[i], wl[i], t, off) > pw_weight(wo[i - 1], wf[i - 1], wl[i - 1], t, off))) {
            uint8_t c8 = wc[i]; wc[i] = wc[i - 1]; wc[i - 1] = c8;
            uint16_t d16 = wd[i]; wd[i] = wd[i - 1]; wd[i - 1] = d16;
            uint32_t a = wo[i]; wo[i] = wo[i - 1]; wo[i - 1] = a;
            a = wf[i]; wf[i] = wf[i - 1]; wf[i - 1] = a;
            a = wl[i]; wl[i] = wl[i - 1]; wl[i - 1] = a;
            --i;
        }
    }
    for (int i = 1; i < L; ++i) {
        if (wf[i] != kPwNone) continue;
        const int ri = (int)(pw_draw(D.seed, t, (uint32_t)p, k++) % (uint32_t)i);
        const int offc = (int)(pw_draw(D.seed, t, (uint32_t)p, k++) % (th.color + 1u)) - (int)th.color / 2;
        const int v = (int)wc[ri] + offc;
        wc[i] = (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v);
        wd[i] = wd[ri];
        const uint32_t occ = (uint32_t)((float)wo[ri] * ((float)(L - i) / (float)L));
        wo[i] = occ > 1u ? occ : 1u;
        wf[i] = t;
        wl[i] = t;
    }
    for (int j = 0; j < L; ++j) {
        const size_t a = pw_slot(S, buf, j, p);
        S.wColor[a] = wc[j];
        S.wDesc[a] = wd[j];
        S.wOcc[a] = wo[j];
        S.wFirst[a] = wf[j];
        S.wLast[a] = wl[j];
    }
    D.kctr[p] = (uint16_t)k;
}

// global resampling from equally spaced pixels (two passes) and the fill of empty dictionary
// slots; one thread per stream (it visits about 4 G pixels)
extern "C" __global__ void pw_k_refresh_global(PawcsDev S, uint32_t t, int buf, int force, int onlyPending,
                                               int useDil) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    PawcsCtl* pc = S.pc;
    if (onlyPending && pc->reset_pending == 0) return;
    const StreamDev& D = S.sd;
    const int G = S.G, L = S.L;
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
            const PwThr th = pw_thresholds(fm[FM_R * D.npx + p], S.unstable[p], S.minColor, S.descOff);
            const size_t a = pw_slot(S, buf, 0, (int)p);
            const uint32_t bc = S.wColor[a], bd = S.wDesc[a];
            const float bw = pw_weight(S.wOcc[a], S.wFirst[a], S.wLast[a], t, off);
            const uint32_t bb = __popc(bd);
            int uninit = 0, g;
            for (g = 0; g < G; ++g) {
                const int w = pc->gdict[g];
                if (w < 0) {
                    uninit = 1;
                    continue;
                }
                if (pw_absdiff(pc->gw_color[w], bc) <= th.color && pw_absdiff(bb, pc->gw_bits[w]) <= th.desc / 4u) break;
            }
            if (g == G) {
                g = G - 1;
                const int w = uninit ? pc->gnext++ : pc->gdict[g];
                pc->gw_color[w] = bc;
                pc->gw_desc[w] = bd;
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
        pc->gw_bits[w] = 0;
        for (size_t i = 0; i < n; ++i) S.gmap[(size_t)w * n + i] = 0.0f;
        pc->gw_weight[w] = 0.0f;
        pc->gdict[g] = w;
    }
    (void)L;
}

// the automatic reset's T(x) := 1 (:1508)
extern "C" __global__ void pw_k_reset_T(PawcsDev S, int buf) {
    if (S.pc->reset_pending == 0) return;
    const StreamDev& D = S.sd;
    float* T = D.fm + (size_t)buf * kNumFloatMaps * D.npx + FM_T * D.npx;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) T[p] = 1.0f;
}

// initial state of a stream's maps (:472-520) and dictionaries
extern "C" __global__ void pw_k_init(PawcsDev S) {
    const StreamDev& D = S.sd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        for (int b = 0; b < 2; ++b) {
            float* f = D.fm + (size_t)b * kNumFloatMaps * D.npx;
            for (int m = 0; m < kNumFloatMaps; ++m) f[m * D.npx + p] = 0.0f;
            f[FM_T * D.npx + p] = kTLower;
            f[FM_R * D.npx + p] = 2.0f;
            f[FM_V * D.npx + p] = kVIncr * 10;
            for (int j = 0; j < S.L; ++j) {
                const size_t a = pw_slot(S, b, j, p);
                S.wColor[a] = 0;
                S.wDesc[a] = 0;
                S.wOcc[a] = 0;
                S.wFirst[a] = kPwNone;
                S.wLast[a] = 0;
            }
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

// last colour and LBSP descriptor of the initialization frame (BackgroundSubtractionUtils.cpp:115-150,
// BackgroundSubtractorLBSP.cpp:26-38: descriptors strictly inside the 2-pixel border)
extern "C" __global__ void pw_k_init_last(PawcsDev S, const uint8_t* img) {
    const StreamDev& D = S.sd;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        const int x = p % D.W, y = p / D.W;
        uint8_t c = 0;
        uint16_t d = 0;
        if (D.roi[p]) {
            c = img[p];
            if (x > 2 && y > 2 && x < D.W - 2 && y < D.H - 2) {
                uint8_t taps[16];
                pw_taps(img, D.W, x, y, taps);
                d = (uint16_t)pw_lbsp(taps, c, D.ctl->lut[c]);
            }
        }
        D.lastCol[p] = c;
        D.lastDesc[p] = d;
    }
}

// camera-motion comparison (:1480-1501), frames t with t % 500 == 0: the background image of the words
// of buffer buf, area-down-sampled like the frame, against the long-term mean of the down-sampled
// frames; one thread per down-sampled pixel writes |LT - BG| (0 outside the fully covered blocks)
extern "C" __global__ void pw_k_motion_bg(PwParams P, int buf) {
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    const int nds = D.dsW * D.dsH;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nds) return;
    if (S.dsRoi[i] != 255) {
        S.dsAbs[i] = 0.0f;
        return;
    }
    const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
    const unsigned long long off = S.pc->lword_offset;
    const int bx = i % D.dsW, by = i / D.dsW;
    // the background image (0 outside the ROI), area-down-sampled
    const uint8_t v = area_resample(D.W, D.H, D.dsW, D.dsH, bx, by, [&](int sx, int sy) {
        const int p = sy * D.W + sx;
        if (!D.roi[p]) return 0;
        float tw = 0.0f, tc = 0.0f;
        for (int j = 0; j < S.L; ++j) {
            const size_t a = pw_slot(S, buf, j, p);
            const float w = pw_weight(S.wOcc[a], S.wFirst[a], S.wLast[a], t, off);
            tc = tc + (float)S.wColor[a] * w;
            tw = tw + w;
        }
        const int r = __float2int_rn(tc / tw);
        return r < 0 ? 0 : r > 255 ? 255 : r;
    });
    S.dsAbs[i] = fabsf(D.dsLT[i] - (float)v);
}

// camera-motion decision: ordered L1 sum, then switch the mode on (during the bootstrap window, ratio
// >= 45) or off (ratio < 45/4) with the local word weight offset (5 / 1000); flags[1] tells the host
// to run refreshModel(1, 1, true), flags[2] carries the new offset. One grayscale channel: the colour
// distance ratio is 0; three channels: the mean colour distortion of pw3_k_motion_bg.
extern "C" __global__ void pw_k_motion_decide(PwParams P) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const PawcsDev& S = P.streams[0];
    const StreamDev& D = S.sd;
    PawcsCtl* pc = S.pc;
    pc->motion_pending = 0;
    if (pc->reset_block) {
        const uint32_t t = (uint32_t)(D.ctl->frame_idx + 1ull);
        const int boot = t <= (uint32_t)kBootWin;
        const int nds = D.dsW * D.dsH;
        float l1 = 0.0f;
        for (int i = 0; i < nds; ++i) l1 = l1 + S.dsAbs[i];
        const float mr = l1 / (float)pc->ds_roi_count;
        float cr = 0.0f;
        if (D.C == 3) {
            // three channels: the ordered sum of the colour distortions (written beside the L1 terms)
            float cs = 0.0f;
            for (int i = 0; i < nds; ++i) cs = cs + S.contrib[i];
            cr = cs / (float)pc->ds_roi_count;
        }
        if (pc->moving_cam && mr < (float)(45 / 4) && cr < (float)(45 / 10 / 4)) {
            pc->lword_offset = (unsigned long long)kBootWin * 2;
            pc->moving_cam = 0;
            pc->motion_pending = 1;
        } else if (boot && !pc->moving_cam && (mr >= 45.0f || cr >= (float)(45 / 10))) {
            pc->lword_offset = 5;
            pc->moving_cam = 1;
            pc->motion_pending = 1;
        }
    }
    P.flags[1] = (unsigned int)pc->motion_pending;
    P.flags[2] = (unsigned int)pc->lword_offset;
}

// background image (:1518-1545) / descriptors (:1547-1594) from the words of buffer buf
extern "C" __global__ void pw_k_background(PawcsDev S, int buf, uint8_t* outCol, uint16_t* outDesc) {
    const StreamDev& D = S.sd;
    const uint32_t t = (uint32_t)D.ctl->frame_idx;
    const unsigned long long off = S.pc->lword_offset;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < D.npx; p += gridDim.x * blockDim.x) {
        if (!D.roi[p]) {
            if (outCol) outCol[p] = 0;
            if (outDesc) outDesc[p] = 0;
            continue;
        }
        float tw = 0.0f, tc = 0.0f, td = 0.0f;
        for (int j = 0; j < S.L; ++j) {
            const size_t a = pw_slot(S, buf, j, p);
            const float w = pw_weight(S.wOcc[a], S.wFirst[a], S.wLast[a], t, off);
            tc = tc + (float)S.wColor[a] * w;
            td = td + (float)S.wDesc[a] * w;
            tw = tw + w;
        }
        if (outCol) {
            const int r = __float2int_rn(tc / tw);
            outCol[p] = (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
        }
        if (outDesc) {
            const int r = __float2int_rn(td / tw);
            outDesc[p] = (uint16_t)(r < 0 ? 0 : r > 65535 ? 65535 : r);
        }
    }
}

}  // namespace lvbgs
