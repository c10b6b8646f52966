// ORACLE (test infrastructure only): C API over the REFERENCE's own BackgroundSubtractorSuBSENSE,
// BackgroundSubtractorPAWCS, BackgroundSubtractorLOBSTER, BackgroundSubtractorViBe and BackgroundSubtractorPBAS
// classes (compiled from the reference's sources by
// oracle/refshim/build_ref.py), with the same signatures and state layouts as the C restatement's
// osub_* / opawcs_* (oracle/oracle.h), so that the tests can run both on the same frames and compare
// every map bit for bit. Built into oracle/_ref/libref.so, which only the CPU tests load.
#include "litiv/video/BackgroundSubtractorLOBSTER.hpp"
#include "litiv/video/BackgroundSubtractorPAWCS.hpp"
#include "litiv/video/BackgroundSubtractorPBAS.hpp"
#include "litiv/video/BackgroundSubtractorSuBSENSE.hpp"
#include "litiv/video/BackgroundSubtractorViBe.hpp"
#include "oracle.h"
#include "philox.h"

namespace {

// ---- the counter-based rand() of the reference (lvshim_rand.h) ----
struct RngCtx {
    uint64_t seed = 0;
    const size_t* frame = nullptr;  // the instance's m_nFrameIdx
    std::vector<uint32_t> k;        // per-pixel draw counters of the current frame
    uint32_t ksent = 0;             // frame-level draws
    void start_frame(size_t npx) {
        k.assign(npx, 0u);
        ksent = 0;
    }
};
thread_local RngCtx* g_rng = nullptr;
thread_local std::string g_last_error;

}  // namespace

int lvshim_rand(size_t px) {
    RngCtx* r = g_rng;
    if (!r || !r->frame) throw std::runtime_error("reference rand() called outside a bridged call");
    uint32_t p32, kk;
    if (px == SIZE_MAX) {
        p32 = OPHILOX_SENTINEL_PX;
        kk = r->ksent++;
    } else {
        if (px >= r->k.size()) throw std::runtime_error("reference rand(): pixel out of range");
        p32 = (uint32_t)px;
        kk = r->k[px]++;
    }
    const uint32_t ctr[4] = {kk >> 2, p32, (uint32_t)*r->frame, 0u};
    const uint32_t key[2] = {(uint32_t)r->seed, (uint32_t)(r->seed >> 32)};
    uint32_t out[4];
    ophilox4x32_10(ctr, key, out);
    return (int)(out[kk & 3u] & 0x7fffffffu);
}

// the draws of BackgroundSubtractorViBe.cpp (lvshim_rand_xy.h): the loop's pixel (x, y) in apply(),
// (x_orig, y_orig) in initialize(); the sentinels (-1) elsewhere
int lvshim_rand_xy(int px, int py, int pxo, int pyo, int width) {
    if (px >= 0 && py >= 0) return lvshim_rand((size_t)py * (size_t)width + (size_t)px);
    if (pxo >= 0 && pyo >= 0) return lvshim_rand((size_t)pyo * (size_t)width + (size_t)pxo);
    return lvshim_rand(SIZE_MAX);
}

namespace {

// runs f with this instance's generator current; reference exceptions become error codes
template <typename F>
int guarded(RngCtx& rng, F&& f) {
    RngCtx* prev = g_rng;
    g_rng = &rng;
    int rc = OSUB_OK;
    try {
        f();
    } catch (const std::exception& e) {
        g_last_error = e.what();
        rc = OSUB_EBADARG;
    }
    g_rng = prev;
    return rc;
}

inline int mat_type(int channels) { return CV_8UC(channels); }

template <typename T>
void append_mat(std::vector<uint8_t>& out, const cv::Mat& m) {
    const size_t n = m.total() * m.elemSize();
    const size_t o = out.size();
    out.resize(o + n);
    for (int y = 0; y < m.rows; ++y) std::memcpy(out.data() + o + (size_t)y * m.cols * m.elemSize(), m.ptr(y), m.cols * m.elemSize());
}

// ---------------------------------------------------------------------------------------------
// SuBSENSE
// ---------------------------------------------------------------------------------------------
struct RefSub : BackgroundSubtractorSuBSENSE {
    RngCtx rng;
    std::vector<uint8_t> exported;
    explicit RefSub(const osub_params& p)
        : BackgroundSubtractorSuBSENSE(p.desc_dist_threshold_offset, p.min_color_dist_threshold, p.bg_samples,
                                       p.required_bg_samples, p.samples_for_moving_avgs, p.rel_lbsp_threshold) {
        rng.seed = p.seed;
        rng.frame = &m_nFrameIdx;
    }
    int W() const { return m_oImgSize.width; }
    int H() const { return m_oImgSize.height; }
    int C() const { return (int)m_nImgChannels; }
    bool inited() const { return m_bInitialized; }

    const void* map(int which, size_t* nbytes) {
        exported.clear();
        const cv::Mat* m = nullptr;
        switch (which) {
            case OSUB_MAP_R: m = &m_oDistThresholdFrame; break;
            case OSUB_MAP_V: m = &m_oVariationModulatorFrame; break;
            case OSUB_MAP_T: m = &m_oUpdateRateFrame; break;
            case OSUB_MAP_DLAST: m = &m_oMeanLastDistFrame; break;
            case OSUB_MAP_DMIN_LT: m = &m_oMeanMinDistFrame_LT; break;
            case OSUB_MAP_DMIN_ST: m = &m_oMeanMinDistFrame_ST; break;
            case OSUB_MAP_RAW_LT: m = &m_oMeanRawSegmResFrame_LT; break;
            case OSUB_MAP_RAW_ST: m = &m_oMeanRawSegmResFrame_ST; break;
            case OSUB_MAP_FIN_LT: m = &m_oMeanFinalSegmResFrame_LT; break;
            case OSUB_MAP_FIN_ST: m = &m_oMeanFinalSegmResFrame_ST; break;
            case OSUB_MAP_UNSTABLE: m = &m_oUnstableRegionMask; break;
            case OSUB_MAP_BLINKS: m = &m_oBlinksFrame; break;
            case OSUB_MAP_LAST_RAW_FG: m = &m_oLastRawFGMask; break;
            case OSUB_MAP_LAST_FG: m = &m_oLastFGMask; break;
            case OSUB_MAP_LAST_FG_DIL_INV: m = &m_oLastFGMask_dilated_inverted; break;
            case OSUB_MAP_LAST_RAW_BLINK: m = &m_oLastRawFGBlinkMask; break;
            case OSUB_MAP_ROI: m = &m_oROI; break;
            case OSUB_MAP_LAST_COLOR: m = &m_oLastColorFrame; break;
            case OSUB_MAP_LAST_DESC: m = &m_oLastDescFrame; break;
            case OSUB_MAP_DS_LT: m = &m_oMeanDownSampledLastDistFrame_LT; break;
            case OSUB_MAP_DS_ST: m = &m_oMeanDownSampledLastDistFrame_ST; break;
            case OSUB_MAP_SAMPLE_COLOR:
                for (const cv::Mat& s : m_voBGColorSamples) append_mat<uint8_t>(exported, s);
                break;
            case OSUB_MAP_SAMPLE_DESC:
                for (const cv::Mat& s : m_voBGDescSamples) append_mat<uint8_t>(exported, s);
                break;
            case OSUB_MAP_LUT: exported.assign(m_anLBSPThreshold_8bitLUT.begin(), m_anLBSPThreshold_8bitLUT.end()); break;
            default: *nbytes = 0; return nullptr;
        }
        if (m) append_mat<uint8_t>(exported, *m);
        *nbytes = exported.size();
        return exported.data();
    }
    void scalars(osub_scalars* s) const {
        std::memset(s, 0, sizeof(*s));
        s->frame_idx = m_nFrameIdx;
        s->frames_since_last_reset = m_nFramesSinceLastReset;
        s->model_reset_cooldown = m_nModelResetCooldown;
        s->auto_model_reset_enabled = m_bAutoModelResetEnabled;
        s->learning_rate_scaling_enabled = m_bLearningRateScalingEnabled;
        s->use_3x3_spread = m_bUse3x3Spread;
        s->median_blur_kernel_size = m_nMedianBlurKernelSize;
        s->lr_lower_cap = m_fCurrLearningRateLowerCap;
        s->lr_upper_cap = m_fCurrLearningRateUpperCap;
        s->last_nonzero_desc_ratio = m_fLastNonZeroDescRatio;
        s->n_relevant_px = m_nTotRelevantPxCount;
        s->orig_roi_px = m_nOrigROIPxCount;
    }
};

// ---------------------------------------------------------------------------------------------
// LOBSTER. Its apply() never advances m_nFrameIdx, so the generator's frame is a count of the apply()
// calls kept here (initialize() and the refreshes before the first apply() are frame 0).
// ---------------------------------------------------------------------------------------------
struct RefLob : BackgroundSubtractorLOBSTER {
    RngCtx rng;
    size_t frames = 0;
    std::vector<uint8_t> exported;
    explicit RefLob(const olob_params& p)
        : BackgroundSubtractorLOBSTER(p.desc_dist_threshold, p.color_dist_threshold, p.bg_samples,
                                      p.required_bg_samples, p.lbsp_threshold_offset, p.rel_lbsp_threshold) {
        rng.seed = p.seed;
        rng.frame = &frames;
    }
    int W() const { return m_oImgSize.width; }
    int H() const { return m_oImgSize.height; }
    int C() const { return (int)m_nImgChannels; }
    bool inited() const { return m_bInitialized; }
    const void* map(int which, size_t* nbytes) {
        exported.clear();
        const cv::Mat* m = nullptr;
        switch (which) {
            case OLOB_MAP_LAST_FG: m = &m_oLastFGMask; break;
            case OLOB_MAP_ROI: m = &m_oROI; break;
            case OLOB_MAP_LAST_COLOR: m = &m_oLastColorFrame; break;
            case OLOB_MAP_LAST_DESC: m = &m_oLastDescFrame; break;
            case OLOB_MAP_SAMPLE_COLOR:
                for (const cv::Mat& s : m_voBGColorSamples) append_mat<uint8_t>(exported, s);
                break;
            case OLOB_MAP_SAMPLE_DESC:
                for (const cv::Mat& s : m_voBGDescSamples) append_mat<uint8_t>(exported, s);
                break;
            case OLOB_MAP_LUT: exported.assign(m_anLBSPThreshold_8bitLUT.begin(), m_anLBSPThreshold_8bitLUT.end()); break;
            default: *nbytes = 0; return nullptr;
        }
        if (m) append_mat<uint8_t>(exported, *m);
        *nbytes = exported.size();
        return exported.data();
    }
    void scalars(olob_scalars* s) const {
        std::memset(s, 0, sizeof(*s));
        s->frames = frames;
        s->n_relevant_px = m_nTotRelevantPxCount;
        s->orig_roi_px = m_nOrigROIPxCount;
    }
};

// ---------------------------------------------------------------------------------------------
// ViBe: BackgroundSubtractorViBe_1ch for single-channel frames, _3ch for three-channel frames (the
// instance is made at initialize()); no frame counter either, so the generator's frame counts apply()
// calls here too
// ---------------------------------------------------------------------------------------------
template <typename B>
struct RefVibeT : B {
    using B::B;
    const std::vector<cv::Mat>& samples() const { return this->m_voBGImg; }
};
struct RefVibe {
    ovibe_params p;
    RngCtx rng;
    size_t frames = 0;
    int W = 0, H = 0, C = 0;
    std::unique_ptr<BackgroundSubtractorViBe> algo;
    std::vector<uint8_t> exported;
    explicit RefVibe(const ovibe_params& q) : p(q) {
        rng.seed = q.seed;
        rng.frame = &frames;
    }
    const std::vector<cv::Mat>& samples() const {
        return C == 1 ? static_cast<const RefVibeT<BackgroundSubtractorViBe_1ch>*>(algo.get())->samples()
                      : static_cast<const RefVibeT<BackgroundSubtractorViBe_3ch>*>(algo.get())->samples();
    }
};

// ---------------------------------------------------------------------------------------------
// PBAS: BackgroundSubtractorPBAS_1ch / _3ch, made at initialize() like ViBe's
// ---------------------------------------------------------------------------------------------
template <typename B>
struct RefPbasT : B {
    using B::B;
    const std::vector<cv::Mat>& colours() const { return this->m_voBGImg; }
    const std::vector<cv::Mat>& grads() const { return this->m_voBGGrad; }
    const cv::Mat& map(int which) const {
        return which == OPBAS_MAP_R ? this->m_oDistThresholdFrame
                                    : which == OPBAS_MAP_T ? this->m_oUpdateRateFrame : this->m_oMeanMinDistFrame;
    }
    float meanGrad() const { return this->m_fFormerMeanGradDist; }
};
struct RefPbas {
    opbas_params p;
    RngCtx rng;
    size_t frames = 0;
    int W = 0, H = 0, C = 0;
    std::unique_ptr<BackgroundSubtractorPBAS> algo;
    std::vector<uint8_t> exported;
    explicit RefPbas(const opbas_params& q) : p(q) {
        rng.seed = q.seed;
        rng.frame = &frames;
    }
    template <typename F>
    auto with(F&& f) const {
        return C == 1 ? f(static_cast<const RefPbasT<BackgroundSubtractorPBAS_1ch>*>(algo.get()))
                      : f(static_cast<const RefPbasT<BackgroundSubtractorPBAS_3ch>*>(algo.get()));
    }
};

// ---------------------------------------------------------------------------------------------
// PAWCS
// ---------------------------------------------------------------------------------------------
struct RefPawcs : BackgroundSubtractorPAWCS {
    RngCtx rng;
    explicit RefPawcs(const opawcs_params& p)
        : BackgroundSubtractorPAWCS(p.desc_dist_threshold_offset, p.min_color_dist_threshold, p.max_words,
                                    p.samples_for_moving_avgs, p.rel_lbsp_threshold) {
        rng.seed = p.seed;
        rng.frame = &m_nFrameIdx;
    }
    int W() const { return m_oImgSize.width; }
    int H() const { return m_oImgSize.height; }
    int C() const { return (int)m_nImgChannels; }
    bool inited() const { return m_bInitialized; }

    // storage index of a global word (its position in the word list), -1 for none
    int pool_index(const GlobalWordBase* g) const {
        if (!g) return -1;
        if (m_nImgChannels == 1) {
            for (size_t i = 0; i < m_voGlobalWordList_1ch.size(); ++i)
                if ((const GlobalWordBase*)&m_voGlobalWordList_1ch[i] == g) return (int)i;
        } else {
            for (size_t i = 0; i < m_voGlobalWordList_3ch.size(); ++i)
                if ((const GlobalWordBase*)&m_voGlobalWordList_3ch[i] == g) return (int)i;
        }
        return -1;
    }
    const GlobalWordBase* pool_word(size_t i) const {
        if (m_nImgChannels == 1) return i < m_voGlobalWordList_1ch.size() ? &m_voGlobalWordList_1ch[i] : nullptr;
        return i < m_voGlobalWordList_3ch.size() ? &m_voGlobalWordList_3ch[i] : nullptr;
    }

    size_t export_bytes(int which) const {
        if (!m_bInitialized) return 0;
        const size_t npx = m_nTotPxCount, C = m_nImgChannels, G = m_nCurrGlobalWords;
        const size_t nw = m_nTotRelevantPxCount * m_nCurrLocalWords;
        const size_t gmap = (size_t)m_oDownSampledFrameSize_GlobalWordLookup.area();
        const size_t nds = (size_t)m_oDownSampledFrameSize_MotionAnalysis.area() * C;
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
            case OPAWCS_MAP_GW_MAP: return G * gmap * 4;
            case OPAWCS_MAP_GLUT: return npx * G;
            case OPAWCS_MAP_GW: return G * 20;
            case OPAWCS_MAP_LW_COLOR: return nw * C;
            case OPAWCS_MAP_LW_DESC: return nw * C * 2;
            case OPAWCS_MAP_LW_OCC: case OPAWCS_MAP_LW_FIRST: case OPAWCS_MAP_LW_LAST: return nw * 8;
            default: return 0;
        }
    }

    int export_map(int which, void* out, size_t bytes) const {
        if (!m_bInitialized) return OSUB_ENOTINIT;
        const size_t need = export_bytes(which);
        if (!need || !out || bytes < need) return OSUB_EBADARG;
        uint8_t* o = (uint8_t*)out;
        std::memset(o, 0, need);
        const cv::Mat* m = nullptr;
        const size_t C = m_nImgChannels, G = m_nCurrGlobalWords, L = m_nCurrLocalWords;
        switch (which) {
            case OPAWCS_MAP_R: m = &m_oDistThresholdFrame; break;
            case OPAWCS_MAP_V: m = &m_oDistThresholdVariationFrame; break;
            case OPAWCS_MAP_T: m = &m_oUpdateRateFrame; break;
            case OPAWCS_MAP_DMIN_LT: m = &m_oMeanMinDistFrame_LT; break;
            case OPAWCS_MAP_DMIN_ST: m = &m_oMeanMinDistFrame_ST; break;
            case OPAWCS_MAP_RAW_LT: m = &m_oMeanRawSegmResFrame_LT; break;
            case OPAWCS_MAP_RAW_ST: m = &m_oMeanRawSegmResFrame_ST; break;
            case OPAWCS_MAP_FIN_LT: m = &m_oMeanFinalSegmResFrame_LT; break;
            case OPAWCS_MAP_FIN_ST: m = &m_oMeanFinalSegmResFrame_ST; break;
            case OPAWCS_MAP_ILLUM: m = &m_oIllumUpdtRegionMask; break;
            case OPAWCS_MAP_UNSTABLE: m = &m_oUnstableRegionMask; break;
            case OPAWCS_MAP_BLINKS: m = &m_oBlinksFrame; break;
            case OPAWCS_MAP_LAST_RAW_FG: m = &m_oLastRawFGMask; break;
            case OPAWCS_MAP_LAST_FG: m = &m_oLastFGMask; break;
            case OPAWCS_MAP_LAST_FG_DIL: m = &m_oLastFGMask_dilated; break;
            case OPAWCS_MAP_LAST_RAW_BLINK: m = &m_oLastRawFGBlinkMask; break;
            case OPAWCS_MAP_ROI: m = &m_oROI; break;
            case OPAWCS_MAP_LAST_COLOR: m = &m_oLastColorFrame; break;
            case OPAWCS_MAP_LAST_DESC: m = &m_oLastDescFrame; break;
            case OPAWCS_MAP_DS_LT: m = &m_oMeanDownSampledLastDistFrame_LT; break;
            case OPAWCS_MAP_DS_ST: m = &m_oMeanDownSampledLastDistFrame_ST; break;
            case OPAWCS_MAP_LUT: std::memcpy(o, m_anLBSPThreshold_8bitLUT.data(), 256); return OSUB_OK;
            case OPAWCS_MAP_GW_MAP: {
                const size_t gmap = (size_t)m_oDownSampledFrameSize_GlobalWordLookup.area();
                for (size_t w = 0; w < G; ++w) {
                    const GlobalWordBase* g = pool_word(w);
                    if (g && !g->oSpatioOccMap.empty())
                        for (int y = 0; y < g->oSpatioOccMap.rows; ++y)
                            std::memcpy(o + (w * gmap + (size_t)y * g->oSpatioOccMap.cols) * 4, g->oSpatioOccMap.ptr(y),
                                        (size_t)g->oSpatioOccMap.cols * 4);
                }
                return OSUB_OK;
            }
            case OPAWCS_MAP_GLUT:
                for (size_t p = 0; p < m_nTotPxCount; ++p) {
                    const auto& lut = m_voPxInfoLUT_PAWCS[p].vpGlobalDictSortLUT;
                    for (size_t j = 0; j < G && j < lut.size(); ++j) o[p * G + j] = (uint8_t)pool_index(lut[j]);
                }
                return OSUB_OK;
            case OPAWCS_MAP_GW:
                for (size_t w = 0; w < G; ++w) {
                    const GlobalWordBase* g = pool_word(w);
                    if (!g) continue;
                    uint8_t* r = o + w * 20;
                    if (C == 1) {
                        const auto& f = ((const GlobalWord_1ch*)g)->oFeature;
                        r[0] = f.anColor[0];
                        std::memcpy(r + 4, f.anDesc.data(), 2);
                    } else {
                        const auto& f = ((const GlobalWord_3ch*)g)->oFeature;
                        std::memcpy(r, f.anColor.data(), 3);
                        std::memcpy(r + 4, f.anDesc.data(), 6);
                    }
                    r[10] = g->nDescBITS;
                    std::memcpy(r + 12, &g->fLatestWeight, 4);
                    int32_t slot = -1;
                    for (size_t s = 0; s < m_vpGlobalWordDict.size(); ++s)
                        if (m_vpGlobalWordDict[s] == g) slot = (int32_t)s;
                    std::memcpy(r + 16, &slot, 4);
                }
                return OSUB_OK;
            case OPAWCS_MAP_LW_COLOR: case OPAWCS_MAP_LW_DESC: case OPAWCS_MAP_LW_OCC: case OPAWCS_MAP_LW_FIRST:
            case OPAWCS_MAP_LW_LAST: {
                const size_t es = which == OPAWCS_MAP_LW_COLOR ? C : which == OPAWCS_MAP_LW_DESC ? 2 * C : 8;
                const size_t nw = m_nTotRelevantPxCount * L;
                for (size_t k = 0; k < nw && k < m_vpLocalWordDict.size(); ++k) {
                    const LocalWordBase* w = m_vpLocalWordDict[k];
                    if (!w) continue;
                    uint8_t* r = o + k * es;
                    if (which == OPAWCS_MAP_LW_OCC) std::memcpy(r, &w->nOccurrences, 8);
                    else if (which == OPAWCS_MAP_LW_FIRST) std::memcpy(r, &w->nFirstOcc, 8);
                    else if (which == OPAWCS_MAP_LW_LAST) std::memcpy(r, &w->nLastOcc, 8);
                    else if (C == 1) {
                        const auto& f = ((const LocalWord_1ch*)w)->oFeature;
                        if (which == OPAWCS_MAP_LW_COLOR) r[0] = f.anColor[0];
                        else std::memcpy(r, f.anDesc.data(), 2);
                    } else {
                        const auto& f = ((const LocalWord_3ch*)w)->oFeature;
                        if (which == OPAWCS_MAP_LW_COLOR) std::memcpy(r, f.anColor.data(), 3);
                        else std::memcpy(r, f.anDesc.data(), 6);
                    }
                }
                return OSUB_OK;
            }
            default: return OSUB_EBADARG;
        }
        size_t off = 0;
        for (int y = 0; y < m->rows; ++y) {
            const size_t rb = (size_t)m->cols * m->elemSize();
            std::memcpy(o + off, m->ptr(y), rb);
            off += rb;
        }
        return OSUB_OK;
    }

    void scalars(opawcs_scalars* s) const {
        std::memset(s, 0, sizeof(*s));
        s->frame_idx = m_nFrameIdx;
        s->frames_since_last_reset = m_nFramesSinceLastReset;
        s->model_reset_cooldown = m_nModelResetCooldown;
        s->lword_weight_offset = m_nLocalWordWeightOffset;
        s->auto_model_reset_enabled = m_bAutoModelResetEnabled;
        s->using_moving_camera = m_bUsingMovingCamera;
        s->median_blur_kernel_size = m_nMedianBlurKernelSize;
        s->n_local_words = (int32_t)m_nCurrLocalWords;
        s->n_global_words = (int32_t)m_nCurrGlobalWords;
        s->last_nonflat_ratio = m_fLastNonFlatRegionRatio;
        s->n_relevant_px = m_nTotRelevantPxCount;
        s->orig_roi_px = m_nOrigROIPxCount;
        s->ds_roi_px = m_nDownSampledROIPxCount;
    }
};

cv::Mat roi_mat(const uint8_t* roi, int W, int H) {
    if (!roi) return cv::Mat();
    return cv::Mat(H, W, CV_8UC1, (void*)roi).clone();
}

}  // namespace

extern "C" {

// message of the last exception the reference threw on this thread
const char* r_last_error() { return g_last_error.c_str(); }

// ---- SuBSENSE: the reference's BackgroundSubtractorSuBSENSE (BackgroundSubtractorSuBSENSE.cpp) ----
void* rsub_create(const osub_params* p) {
    // the reference's constructor fixes the LBSP offset (0) and the default median size (9)
    if (p->lbsp_threshold_offset != 0 || p->default_median_blur_kernel_size != 9) return nullptr;
    try {
        return new RefSub(*p);
    } catch (...) {
        return nullptr;
    }
}
void rsub_destroy(void* h) { delete (RefSub*)h; }
int rsub_initialize(void* h, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    RefSub* o = (RefSub*)h;
    o->rng.start_frame((size_t)W * H);
    cv::Mat m(H, W, mat_type(C), (void*)img);
    const cv::Mat r = roi_mat(roi, W, H);
    // initialize() runs as frame 0 (m_nFrameIdx is reset to 0 by initialize_common before any draw)
    return guarded(o->rng, [&] { o->initialize(m, r); });
}
int rsub_apply(void* h, const uint8_t* img, uint8_t* mask, double lr) {
    RefSub* o = (RefSub*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    o->rng.start_frame((size_t)o->W() * o->H());
    cv::Mat m(o->H(), o->W(), mat_type(o->C()), (void*)img);
    cv::Mat out(o->H(), o->W(), CV_8UC1, (void*)mask);
    return guarded(o->rng, [&] { o->apply(m, out, lr); });
}
int rsub_refresh_model(void* h, float frac, int force) {
    RefSub* o = (RefSub*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    return guarded(o->rng, [&] { o->refreshModel(frac, force != 0); });
}
int rsub_get_background(void* h, uint8_t* out) {
    RefSub* o = (RefSub*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rsub_get_background_descriptors(void* h, uint16_t* out) {
    RefSub* o = (RefSub*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundDescriptorsImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rsub_set_roi(void* h, const uint8_t* roi, int W, int H) {
    RefSub* o = (RefSub*)h;
    cv::Mat r = roi_mat(roi, W, H);
    o->rng.start_frame((size_t)W * H);
    // setROI re-initializes from the background image when initialized (frame 0 again)
    return guarded(o->rng, [&] { o->setROI(r); });
}
void rsub_set_automatic_model_reset(void* h, int enabled) { ((RefSub*)h)->setAutomaticModelReset(enabled != 0); }
const void* rsub_map(void* h, int which, size_t* nbytes) { return ((RefSub*)h)->map(which, nbytes); }
void rsub_get_scalars(void* h, osub_scalars* s) { ((RefSub*)h)->scalars(s); }

// ---- PAWCS: the reference's BackgroundSubtractorPAWCS (BackgroundSubtractorPAWCS.cpp) ----
void* rpawcs_create(const opawcs_params* p) {
    if (p->lbsp_threshold_offset != 0 || p->default_median_blur_kernel_size != 9) return nullptr;
    try {
        return new RefPawcs(*p);
    } catch (...) {
        return nullptr;
    }
}
void rpawcs_destroy(void* h) { delete (RefPawcs*)h; }
int rpawcs_initialize(void* h, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    RefPawcs* o = (RefPawcs*)h;
    o->rng.start_frame((size_t)W * H);
    cv::Mat m(H, W, mat_type(C), (void*)img);
    const cv::Mat r = roi_mat(roi, W, H);
    return guarded(o->rng, [&] { o->initialize(m, r); });
}
int rpawcs_apply(void* h, const uint8_t* img, uint8_t* mask, double lr) {
    RefPawcs* o = (RefPawcs*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    o->rng.start_frame((size_t)o->W() * o->H());
    cv::Mat m(o->H(), o->W(), mat_type(o->C()), (void*)img);
    cv::Mat out(o->H(), o->W(), CV_8UC1, (void*)mask);
    return guarded(o->rng, [&] { o->apply(m, out, lr); });
}
int rpawcs_refresh_model(void* h, size_t base_occ, float decr, int force) {
    RefPawcs* o = (RefPawcs*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    return guarded(o->rng, [&] { o->refreshModel(base_occ, decr, force != 0); });
}
int rpawcs_get_background(void* h, uint8_t* out) {
    RefPawcs* o = (RefPawcs*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rpawcs_get_background_descriptors(void* h, uint16_t* out) {
    RefPawcs* o = (RefPawcs*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundDescriptorsImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rpawcs_set_roi(void* h, const uint8_t* roi, int W, int H) {
    RefPawcs* o = (RefPawcs*)h;
    cv::Mat r = roi_mat(roi, W, H);
    o->rng.start_frame((size_t)W * H);
    return guarded(o->rng, [&] { o->setROI(r); });
}
void rpawcs_set_automatic_model_reset(void* h, int enabled) { ((RefPawcs*)h)->setAutomaticModelReset(enabled != 0); }
int rpawcs_export(void* h, int which, void* out, size_t bytes) { return ((RefPawcs*)h)->export_map(which, out, bytes); }
size_t rpawcs_export_bytes(void* h, int which) { return ((RefPawcs*)h)->export_bytes(which); }
void rpawcs_get_scalars(void* h, opawcs_scalars* s) { ((RefPawcs*)h)->scalars(s); }

// ---- LOBSTER: the reference's BackgroundSubtractorLOBSTER (BackgroundSubtractorLOBSTER.cpp) ----
void* rlob_create(const olob_params* p) {
    // the reference's constructor fixes the default median size (9)
    if (p->default_median_blur_kernel_size != 9) return nullptr;
    try {
        return new RefLob(*p);
    } catch (...) {
        return nullptr;
    }
}
void rlob_destroy(void* h) { delete (RefLob*)h; }
int rlob_initialize(void* h, const uint8_t* img, int W, int H, int C, const uint8_t* roi) {
    RefLob* o = (RefLob*)h;
    o->frames = 0;
    o->rng.start_frame((size_t)W * H);
    cv::Mat m(H, W, mat_type(C), (void*)img);
    const cv::Mat r = roi_mat(roi, W, H);
    return guarded(o->rng, [&] { o->initialize(m, r); });
}
int rlob_apply(void* h, const uint8_t* img, uint8_t* mask, double lr) {
    RefLob* o = (RefLob*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    ++o->frames;
    o->rng.start_frame((size_t)o->W() * o->H());
    cv::Mat m(o->H(), o->W(), mat_type(o->C()), (void*)img);
    cv::Mat out(o->H(), o->W(), CV_8UC1, (void*)mask);
    return guarded(o->rng, [&] { o->apply(m, out, lr); });
}
int rlob_refresh_model(void* h, float frac, int force) {
    RefLob* o = (RefLob*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    return guarded(o->rng, [&] { o->refreshModel(frac, force != 0); });
}
int rlob_get_background(void* h, uint8_t* out) {
    RefLob* o = (RefLob*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rlob_get_background_descriptors(void* h, uint16_t* out) {
    RefLob* o = (RefLob*)h;
    if (!o->inited()) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->getBackgroundDescriptorsImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
int rlob_set_roi(void* h, const uint8_t* roi, int W, int H) {
    RefLob* o = (RefLob*)h;
    cv::Mat r = roi_mat(roi, W, H);
    // setROI re-initializes from the background image when initialized: frame 0 again
    o->frames = 0;
    o->rng.start_frame((size_t)W * H);
    return guarded(o->rng, [&] { o->setROI(r); });
}
const void* rlob_map(void* h, int which, size_t* nbytes) { return ((RefLob*)h)->map(which, nbytes); }
void rlob_get_scalars(void* h, olob_scalars* s) { ((RefLob*)h)->scalars(s); }

// ---- ViBe: the reference's BackgroundSubtractorViBe_1ch / _3ch (BackgroundSubtractorViBe.cpp) ----
void* rvibe_create(const ovibe_params* p) {
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return nullptr;
    return new RefVibe(*p);
}
void rvibe_destroy(void* h) { delete (RefVibe*)h; }
int rvibe_initialize(void* h, const uint8_t* img, int W, int H, int C) {
    RefVibe* o = (RefVibe*)h;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED;
    o->frames = 0;
    o->rng.start_frame((size_t)W * H);
    return guarded(o->rng, [&] {
        if (C == 1)
            o->algo.reset(new RefVibeT<BackgroundSubtractorViBe_1ch>(o->p.color_dist_threshold, o->p.bg_samples,
                                                                     o->p.required_bg_samples));
        else
            o->algo.reset(new RefVibeT<BackgroundSubtractorViBe_3ch>(o->p.color_dist_threshold, o->p.bg_samples,
                                                                     o->p.required_bg_samples));
        o->W = W;
        o->H = H;
        o->C = C;
        o->algo->initialize(cv::Mat(H, W, mat_type(C), (void*)img));
    });
}
int rvibe_apply(void* h, const uint8_t* img, uint8_t* mask, double lr) {
    RefVibe* o = (RefVibe*)h;
    if (!o->algo) return OSUB_ENOTINIT;
    ++o->frames;
    o->rng.start_frame((size_t)o->W * o->H);
    cv::Mat m(o->H, o->W, mat_type(o->C), (void*)img);
    cv::Mat out(o->H, o->W, CV_8UC1, (void*)mask);
    return guarded(o->rng, [&] { o->algo->apply(m, out, lr); });
}
int rvibe_get_background(void* h, uint8_t* out) {
    RefVibe* o = (RefVibe*)h;
    if (!o->algo) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->algo->getBackgroundImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
const void* rvibe_samples(void* h, size_t* nbytes) {
    RefVibe* o = (RefVibe*)h;
    o->exported.clear();
    if (!o->algo) {
        *nbytes = 0;
        return nullptr;
    }
    for (const cv::Mat& s : o->samples()) append_mat<uint8_t>(o->exported, s);
    *nbytes = o->exported.size();
    return o->exported.data();
}

// ---- PBAS: the reference's BackgroundSubtractorPBAS_1ch / _3ch (BackgroundSubtractorPBAS.cpp) ----
void* rpbas_create(const opbas_params* p) {
    if (!p || p->bg_samples == 0 || p->required_bg_samples > p->bg_samples) return nullptr;
    return new RefPbas(*p);
}
void rpbas_destroy(void* h) { delete (RefPbas*)h; }
int rpbas_initialize(void* h, const uint8_t* img, int W, int H, int C) {
    RefPbas* o = (RefPbas*)h;
    if (C != 1 && C != 3) return OSUB_EUNSUPPORTED;
    o->frames = 0;
    o->rng.start_frame((size_t)W * H);
    return guarded(o->rng, [&] {
        // one instance per channel count, initialized again like a user's (which keeps its former mean
        // gradient distance)
        if (o->algo && o->C == C) {
        } else if (C == 1) {
            o->algo.reset(new RefPbasT<BackgroundSubtractorPBAS_1ch>(o->p.color_dist_threshold, o->p.update_rate,
                                                                     o->p.bg_samples, o->p.required_bg_samples));
        } else {
            o->algo.reset(new RefPbasT<BackgroundSubtractorPBAS_3ch>(o->p.color_dist_threshold, o->p.update_rate,
                                                                     o->p.bg_samples, o->p.required_bg_samples));
        }
        o->W = W;
        o->H = H;
        o->C = C;
        o->algo->initialize(cv::Mat(H, W, mat_type(C), (void*)img));
    });
}
int rpbas_apply(void* h, const uint8_t* img, uint8_t* mask, double lr) {
    RefPbas* o = (RefPbas*)h;
    if (!o->algo) return OSUB_ENOTINIT;
    ++o->frames;
    o->rng.start_frame((size_t)o->W * o->H);
    cv::Mat m(o->H, o->W, mat_type(o->C), (void*)img);
    cv::Mat out(o->H, o->W, CV_8UC1, (void*)mask);
    return guarded(o->rng, [&] { o->algo->apply(m, out, lr); });
}
int rpbas_get_background(void* h, uint8_t* out) {
    RefPbas* o = (RefPbas*)h;
    if (!o->algo) return OSUB_ENOTINIT;
    cv::Mat bg;
    const int rc = guarded(o->rng, [&] { o->algo->getBackgroundImage(bg); });
    if (rc == OSUB_OK) std::memcpy(out, bg.data, bg.total() * bg.elemSize());
    return rc;
}
const void* rpbas_map(void* h, int which, size_t* nbytes) {
    RefPbas* o = (RefPbas*)h;
    o->exported.clear();
    if (!o->algo || which == OPBAS_MAP_GRAD) {
        *nbytes = 0;
        return nullptr;
    }
    o->with([&](auto* a) {
        if (which == OPBAS_MAP_SAMPLE_COLOR)
            for (const cv::Mat& s : a->colours()) append_mat<uint8_t>(o->exported, s);
        else if (which == OPBAS_MAP_SAMPLE_GRAD)
            for (const cv::Mat& s : a->grads()) append_mat<uint8_t>(o->exported, s);
        else
            append_mat<uint8_t>(o->exported, a->map(which));
        return 0;
    });
    *nbytes = o->exported.size();
    return o->exported.data();
}
float rpbas_mean_grad(void* h) {
    RefPbas* o = (RefPbas*)h;
    return o->algo ? o->with([](auto* a) { return a->meanGrad(); }) : 0.0f;
}

}  // extern "C"
