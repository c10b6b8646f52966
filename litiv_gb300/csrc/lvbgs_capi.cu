// C-ABI of the SuBSENSE CUDA path (include/lvbgs.h): handle management, parameter and input
// validation (the reference's lvAssert_ checks), device allocation of the model, staging of
// host/device frames, and the cooperative launch of the tick kernel for one or many streams.
#include <cuda_runtime.h>

#include <chrono>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/lvbgs.h"
#include "lobster_internal.h"
#include "lvbgs_internal.h"
#include "pawcs_internal.h"

namespace lvbgs {
extern "C" __global__ void lvbgs_k_eval(TickParams P);
extern "C" __global__ void lvbgs_k_longscan(TickParams P);
extern "C" __global__ void lvbgs_k_resolve(TickParams P, unsigned long long dsTotal, const unsigned long long* dsBase);
extern "C" __global__ void lvbgs_k_repair(TickParams P);
extern "C" __global__ void lvbgs_k_commit(TickParams P);
extern "C" __global__ void lvbgs_k_runs(TickParams P);
extern "C" __global__ void lvbgs_k_vunion(TickParams P);
extern "C" __global__ void lvbgs_k_holes(TickParams P);
extern "C" __global__ void lvbgs_k_combine(TickParams P);
extern "C" __global__ void lvbgs_k_hcount(TickParams P);
extern "C" __global__ void lvbgs_k_median(TickParams P);
extern "C" __global__ void lvbgs_k_epilogue(TickParams P);
extern "C" __global__ void lvbgs_k_dilate(TickParams P);
extern "C" __global__ void lvbgs_k_reset(TickParams P);
extern "C" __global__ void lvbgs_k_close(TickParams P);
extern "C" __global__ void lvbgs_init_maps(StreamDev S, const uint8_t* img, float tLo);
extern "C" __global__ void lvbgs_refresh(StreamDev S, uint32_t frame, int start, int nref, int force, int lastBuf);
extern "C" __global__ void lvbgs_background(StreamDev S, uint8_t* outCol, uint16_t* outDesc);
extern "C" __global__ void lvbgs_unpack_samples(StreamDev S, uint8_t* col, uint16_t* desc);
extern "C" __global__ void lvbgs_pack_samples(StreamDev S, const uint8_t* col, const uint16_t* desc);
extern "C" __global__ void lvbgs_init_tables();
extern "C" __global__ void lvbgs_lbsp_dense(const uint8_t* img, int W, int H, int C, int absThr, float rel,
                                            unsigned int off, uint16_t* desc);
// PAWCS (pawcs_kernels.cu)
extern "C" __global__ void pw_k_local(PwParams P);
extern "C" __global__ void pw_k_illum(PwParams P);
extern "C" __global__ void pw_k_cells(PwParams P, int final);
extern "C" __global__ void pw_k_nbr(PwParams P);
extern "C" __global__ void pw_k_replace(PwParams P);
extern "C" __global__ void pw_k_nbr_loops(PwParams P);
extern "C" __global__ void pw_k_dirty(PwParams P);
extern "C" __global__ void pw_k_round_end(PwParams P);
extern "C" __global__ void pw_k_commit(PwParams P);
extern "C" __global__ void pw_k_weights(PwParams P);
extern "C" __global__ void pw_k_gw_recalc(PwParams P);
extern "C" __global__ void pw_k_gw_decay(PwParams P, double* rowsum);
extern "C" __global__ void pw_k_gw_blur(PwParams P, const double* rowsum);
extern "C" __global__ void pw_k_gw_sort(PwParams P);
extern "C" __global__ void pw_k_lut_sort(PwParams P, int mode);
extern "C" __global__ void pw_k_blink_close(PwParams P);
extern "C" __global__ void pw_k_epilogue(PwParams P);
extern "C" __global__ void pw_k_ds(PwParams P);
extern "C" __global__ void pw_k_reset_decide(PwParams P);
extern "C" __global__ void pw_k_motion_bg(PwParams P, int buf);
extern "C" __global__ void pw_k_motion_decide(PwParams P);
extern "C" __global__ void pw_k_compact_count(PwParams P, int mode);
extern "C" __global__ void pw_k_compact_offsets(PwParams P, int ncat);
extern "C" __global__ void pw_k_compact_scatter(PwParams P, int mode);
extern "C" __global__ void pw_k_close(PwParams P);
extern "C" __global__ void pw_k_refresh_local(PawcsDev S, uint32_t t, int buf, int baseOcc, float decr, int force,
                                              int onlyPending, int useDil);
extern "C" __global__ void pw_k_refresh_global(PawcsDev S, uint32_t t, int buf, int force, int onlyPending, int useDil);
extern "C" __global__ void pw_k_reset_T(PawcsDev S, int buf);
extern "C" __global__ void pw_k_init(PawcsDev S);
extern "C" __global__ void pw_k_init_last(PawcsDev S, const uint8_t* img);
extern "C" __global__ void pw_k_background(PawcsDev S, int buf, uint8_t* outCol, uint16_t* outDesc);
// PAWCS, three channels (pawcs3_kernels.cu)
extern "C" __global__ void pw3_k_local(PwParams P);
extern "C" __global__ void pw3_k_gscan_seg(PwParams P);
extern "C" __global__ void pw3_k_gscan_walk(PwParams P);
extern "C" __global__ void pw3_k_gscan_fix(PwParams P);
extern "C" __global__ void pw3_k_gscan_fix_walked(PwParams P);
extern "C" __global__ void pw3_k_dirty(PwParams P);
extern "C" __global__ void pw3_k_later(PwParams P);
extern "C" __global__ void pw3_k_commit(PwParams P);
extern "C" __global__ void pw3_k_ds(PwParams P);
extern "C" __global__ void pw3_k_motion_bg(PwParams P, int buf);
extern "C" __global__ void pw3_k_refresh_local(PawcsDev S, uint32_t t, int buf, int baseOcc, float decr, int force,
                                               int onlyPending, int useDil);
extern "C" __global__ void pw3_k_refresh_global(PawcsDev S, uint32_t t, int buf, int force, int onlyPending, int useDil);
extern "C" __global__ void pw3_k_init(PawcsDev S);
extern "C" __global__ void pw3_k_init_last(PawcsDev S, const uint8_t* img);
extern "C" __global__ void pw3_k_background(PawcsDev S, int buf, uint8_t* outCol, uint16_t* outDesc);
}  // namespace lvbgs

using namespace lvbgs;

namespace {

std::mutex g_err_mu;
std::string g_err;

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// work area of one launch: counters, barrier, repair lists, stream descriptor table
struct Workspace {
    TickWork* work = nullptr;
    StreamDev* d_streams = nullptr;
    unsigned long long* d_dsBase = nullptr;
    unsigned long long* lists = nullptr;  // 4 lists of `cap` entries
    size_t cap = 0;
    int nStreamsCap = 0;
    int repairDiv = 1;  // the repair kernel's cooperative grid: 1/repairDiv of the co-resident blocks
    std::vector<StreamDev> h_streams;
    std::vector<unsigned long long> h_dsBase;
    // optional per-kernel timing: a ring of kTimedKernels+1 events per tick
    std::vector<cudaEvent_t> tev;
    int tevTicks = 0, tevNext = 0, tevRecorded = 0;
    void free_events() {
        for (cudaEvent_t e : tev) cudaEventDestroy(e);
        tev.clear();
        tevTicks = tevNext = tevRecorded = 0;
    }
    void release() {
        free_events();
        cudaFree(work);
        cudaFree(d_streams);
        cudaFree(d_dsBase);
        cudaFree(lists);
        *this = Workspace();
    }
    cudaError_t ensure(size_t px, int nStreams) {
        cudaError_t e = cudaSuccess;
        if (!work && (e = cudaMalloc(&work, sizeof(TickWork))) != cudaSuccess) return e;
        if (nStreams > nStreamsCap) {
            cudaFree(d_streams);
            cudaFree(d_dsBase);
            d_streams = nullptr;
            d_dsBase = nullptr;
            const int n = std::max(nStreams, 8);
            if ((e = cudaMalloc(&d_streams, sizeof(StreamDev) * n)) != cudaSuccess) return e;
            if ((e = cudaMalloc(&d_dsBase, sizeof(unsigned long long) * (n + 1))) != cudaSuccess) return e;
            nStreamsCap = n;
        }
        if (px > cap) {
            cudaFree(lists);
            lists = nullptr;
            if ((e = cudaMalloc(&lists, sizeof(unsigned long long) * px * 4)) != cudaSuccess) {
                cap = 0;
                return e;
            }
            cap = px;
        }
        return e;
    }
};

}  // namespace

// a PAWCS frame step in flight: its stream, launch parameters and the stage of its host waits (0: the
// fixed-point rounds, 1: the camera-motion decision, 2: the end of the frame)
struct PwStep {
    cudaStream_t st = nullptr;
    PwParams P{}, PR{};
    int enq = 0, maxRounds = 64, stage = 0;
    uint8_t* mask = nullptr;
    bool devMask = false, active = false;
};

struct lvbgs_ctx {
    lvbgs_algo algo;
    lvbgs_params prm;
    int device = 0;
    std::string err;
    bool initialized = false;
    int roiW = 0, roiH = 0;  // size of the ROI kept in `roi` (the last validated one, or set before initialize)
    bool spilled = false;
    int W = 0, H = 0, C = 0;
    size_t npx = 0;
    std::vector<uint8_t> roi;
    size_t n_rel = 0, orig_roi = 0;
    // device memory: one block, persistent state first (the spill image), then scratch
    uint8_t* dmem = nullptr;
    size_t persistBytes = 0, totalBytes = 0;
    StreamDev sd{};  // host copy of the descriptor (device pointers)
    uint8_t* d_frame = nullptr;
    uint8_t* d_mask = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t aux[3] = {nullptr, nullptr, nullptr};   // streams of a split batch's further groups (lazily created)
    cudaEvent_t evFork = nullptr, evJoin[3] = {nullptr, nullptr, nullptr};  // fork / joins of a split batch
    Workspace ws;       // single-stream launches
    Workspace batchWs;  // batched launches led by this handle
    // PAWCS (algo == LVBGS_ALGO_PAWCS): device descriptor, host mirrors and launch scratch
    PawcsDev pd{};
    PawcsDev* d_pd = nullptr;
    StreamDev* d_sd = nullptr;
    TickWork* d_work = nullptr;
    unsigned int* d_flags = nullptr;
    double* d_rowsum = nullptr;
    unsigned int* h_flags = nullptr;  // pinned
    unsigned long long pw_frames = 0;
    unsigned long long pw_offset = 1000;
    int pw_rounds_last = 0;
    double pw_host_ms[5] = {0, 0, 0, 0, 0};  // last PAWCS frame: lvbgs_debug_pawcs_host_timing
    PwStep pws;  // the PAWCS frame step in flight (pw_begin / pw_advance)
    cudaEvent_t evPw = nullptr;  // fork / join of the handle's PAWCS step in a batch
    int dbg_fault = 0;  // one-shot fault injection of the next frame step (lvbgs_debug_inject_fault)
    LobState* lob = nullptr;  // LOBSTER and ViBe (LVBGS_ALGO_LOBSTER / _VIBE): the stream's device state
};

namespace {

lvbgs_status fail(lvbgs_handle h, lvbgs_status st, const std::string& msg) {
    if (h) h->err = msg;
    std::lock_guard<std::mutex> lk(g_err_mu);
    g_err = msg;
    return st;
}
lvbgs_status cuda_fail(lvbgs_handle h, cudaError_t e, const char* what) {
    const lvbgs_status st = (e == cudaErrorMemoryAllocation) ? LVBGS_OOM : LVBGS_DEVICE_ERROR;
    return fail(h, st, std::string(what) + ": " + cudaGetErrorString(e));
}
#define LV_CUDA(h, call, what)                          \
    do {                                                \
        cudaError_t e_ = (call);                        \
        if (e_ != cudaSuccess) return cuda_fail(h, e_, what); \
    } while (0)

bool is_device_ptr(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}
// a mask destination the kernels can write themselves: device or managed memory, or page-locked host
// memory registered with CUDA and mapped at the same address (unified addressing), which the
// post-processing kernel then writes over the host link while it runs, with no copy after the frame
// step; pageable host memory is written by a copy from a device staging buffer
bool mask_writable_by_device(const void* p) {
    if (!p) return false;
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return true;
    return a.type == cudaMemoryTypeHost && a.devicePointer == p;
}

// layout of one stream's device block
struct Layout {
    size_t off[32];
    size_t persist, total;
};
enum {
    L_CTL = 0, L_FM, L_UNST, L_LASTCOL, L_LASTDESC, L_SD, L_SC, L_ROI, L_BLINKS, L_LASTRAWFG, L_LASTFG, L_DILINV,
    L_LASTRAWBLINK, L_KCTR, L_DSLT, L_DSST,
    // scratch (not spilled)
    L_STAMPD, L_STAMPR, L_GOODREC, L_BITS, L_HCOUNT, L_LABEL, L_INTENT, L_FRAME, L_MASK, L_COUNT
};
Layout make_layout(int W, int H, int C, size_t N) {
    const size_t npx = (size_t)W * H;
    const size_t nds = (size_t)(W / 8) * (H / 8) * C;
    size_t sz[L_COUNT];
    sz[L_CTL] = sizeof(StreamCtl);
    sz[L_FM] = 2 * kNumFloatMaps * npx * 4;
    sz[L_UNST] = 2 * npx;
    sz[L_LASTCOL] = 2 * npx * C;
    sz[L_LASTDESC] = 2 * npx * C * 2;
    sz[L_SD] = N * npx * (C == 3 ? 8 : 2);
    sz[L_SC] = N * npx;
    sz[L_ROI] = sz[L_BLINKS] = sz[L_LASTRAWFG] = sz[L_LASTFG] = sz[L_DILINV] = sz[L_LASTRAWBLINK] = npx;
    sz[L_KCTR] = npx * 2;
    sz[L_DSLT] = sz[L_DSST] = std::max<size_t>(nds, 1) * 4;
    sz[L_STAMPD] = sz[L_STAMPR] = npx * 4;
    sz[L_GOODREC] = npx * 16;
    sz[L_BITS] = bit_planes_bytes(W, H);
    sz[L_HCOUNT] = npx;
    sz[L_LABEL] = sz[L_INTENT] = npx * 4;
    sz[L_FRAME] = npx * C;
    sz[L_MASK] = npx;
    Layout L;
    size_t o = 0;
    for (int i = 0; i < L_COUNT; ++i) {
        if (i == L_STAMPD) L.persist = o;
        L.off[i] = o;
        o += align256(sz[i]);
    }
    L.total = o;
    return L;
}

void fill_pointers(lvbgs_ctx* h, const Layout& L) {
    StreamDev& S = h->sd;
    uint8_t* b = h->dmem;
    S.ctl = (StreamCtl*)(b + L.off[L_CTL]);
    S.fm = (float*)(b + L.off[L_FM]);
    S.unst = b + L.off[L_UNST];
    S.lastCol = b + L.off[L_LASTCOL];
    S.lastDesc = (uint16_t*)(b + L.off[L_LASTDESC]);
    S.sD = b + L.off[L_SD];
    S.sC = b + L.off[L_SC];
    S.roi = b + L.off[L_ROI];
    S.blinks = b + L.off[L_BLINKS];
    S.lastRawFG = b + L.off[L_LASTRAWFG];
    S.lastFG = b + L.off[L_LASTFG];
    S.dilInv = b + L.off[L_DILINV];
    S.lastRawBlink = b + L.off[L_LASTRAWBLINK];
    S.kctr = (uint16_t*)(b + L.off[L_KCTR]);
    S.dsLT = (float*)(b + L.off[L_DSLT]);
    S.dsST = (float*)(b + L.off[L_DSST]);
    S.stampD = (uint32_t*)(b + L.off[L_STAMPD]);
    S.stampR = (uint32_t*)(b + L.off[L_STAMPR]);
    S.goodRec = (uint4*)(b + L.off[L_GOODREC]);
    S.bits = (uint32_t*)(b + L.off[L_BITS]);
    S.hcount = b + L.off[L_HCOUNT];
    S.label = (int*)(b + L.off[L_LABEL]);
    S.intent = (uint32_t*)(b + L.off[L_INTENT]);
    h->d_frame = b + L.off[L_FRAME];
    h->d_mask = b + L.off[L_MASK];
}

void fill_geometry(lvbgs_ctx* h) {
    StreamDev& S = h->sd;
    S.W = h->W;
    S.H = h->H;
    S.C = h->C;
    S.npx = (int)h->npx;
    S.tilesX = (h->W + kTileW - 1) / kTileW;
    S.tilesY = (h->H + kTileH - 1) / kTileH;
    S.nTiles = S.tilesX * S.tilesY;
    S.tileBase = 0;
    S.rowWords = (h->W + 31) / 32;
    S.segBase = 0;
    S.nSegs = (h->H + kMedSegRows - 1) / kMedSegRows;
    S.dsW = h->W / 8;
    S.dsH = h->H / 8;
    S.N = (int)h->prm.bg_samples;
    S.nreq = (int)h->prm.required_bg_samples;
    S.minColor = (int)h->prm.min_color_dist_threshold;
    S.descOff = (int)h->prm.desc_dist_threshold_offset;
    S.stabColorOff = (int)(h->prm.min_color_dist_threshold / 5);
    S.nmv = (int)h->prm.samples_for_moving_avgs;
    S.relThr = h->prm.rel_lbsp_threshold;
    S.lbspOff = (unsigned)h->prm.lbsp_threshold_offset;
    S.seed = h->prm.seed;
    S.nMagic = ((1ull << 40) + S.N - 1) / (unsigned long long)S.N;
}

constexpr int kTimedKernels = 15;  // kernels of one frame step, in launch order
int g_coop_blocks_per_sm = -1, g_sm_count = 0;
std::mutex g_occ_mu;
cudaError_t coop_grid(int* maxBlocks) {
    std::lock_guard<std::mutex> lk(g_occ_mu);
    if (g_coop_blocks_per_sm < 0) {
        int dev = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e != cudaSuccess) return e;
        if ((e = cudaDeviceGetAttribute(&g_sm_count, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
        if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_coop_blocks_per_sm, lvbgs_k_repair, kThreads, 0)) !=
            cudaSuccess)
            return e;
    }
    *maxBlocks = g_coop_blocks_per_sm * g_sm_count;
    return cudaSuccess;
}

// enqueue one tick over the n streams described in hS (tileBase etc. filled here); hDs holds n+1
// entries. Both are host arrays the descriptor uploads read from (pinned for ticks in flight).
lvbgs_status launch_tick(lvbgs_handle errh, Workspace& ws, int n, cudaStream_t st, StreamDev* hS,
                         unsigned long long* hDs) {
    int totalTiles = 0, totalRows = 0, totalSegs = 0, maxW = 0;
    size_t totalPx = 0;
    unsigned long long ds = 0;
    for (int i = 0; i < n; ++i) {
        StreamDev& S = hS[i];
        S.tileBase = totalTiles;
        S.rowBase = totalRows;
        S.segBase = totalSegs;
        totalTiles += S.nTiles;
        totalRows += S.H;
        totalSegs += S.nSegs;
        maxW = std::max(maxW, S.W);
        totalPx += (size_t)S.npx;
        hDs[i] = ds;
        // only streams with the frame-level analysis enabled down-sample
        if (S.lrScaling) ds += (unsigned long long)S.dsW * S.dsH;
    }
    hDs[n] = ds;
    LV_CUDA(errh, ws.ensure(totalPx, n), "workspace allocation");
    LV_CUDA(errh, cudaMemcpyAsync(ws.d_streams, hS, sizeof(StreamDev) * n, cudaMemcpyHostToDevice, st),
            "descriptor upload");
    LV_CUDA(errh, cudaMemcpyAsync(ws.d_dsBase, hDs, sizeof(unsigned long long) * (n + 1),
                                  cudaMemcpyHostToDevice, st),
            "descriptor upload");
    LV_CUDA(errh, cudaMemsetAsync(ws.work, 0, sizeof(TickWork), st), "work reset");
    int maxBlocks = 0;
    LV_CUDA(errh, coop_grid(&maxBlocks), "occupancy query");
    if (maxBlocks <= 0) return fail(errh, LVBGS_DEVICE_ERROR, "repair kernel cannot be resident on this device");
    TickParams P;
    // one-shot fault injection of the lead handle (lvbgs_debug_inject_fault): waits that give up
    const int fault = errh ? errh->dbg_fault : 0;
    if (errh) errh->dbg_fault = 0;
    P.dbgFault = fault;
    P.barrierNs = fault == LVBGS_FAULT_BARRIER_TIMEOUT ? kDebugBarrierNs : kBarrierNs;
    P.maxRepairIters = fault == LVBGS_FAULT_REPAIR_LIMIT ? 0 : kRepairIterLimit;
    P.streams = ws.d_streams;
    P.nStreams = n;
    P.totalTiles = totalTiles;
    P.totalRows = totalRows;
    P.work = ws.work;
    P.dlist[0] = ws.lists;
    P.dlist[1] = ws.lists + ws.cap;
    P.rlist[0] = ws.lists + 2 * ws.cap;
    P.rlist[1] = ws.lists + 3 * ws.cap;
    P.listCap = (unsigned)std::min<size_t>(ws.cap, 0xffffffffu);
    P.totalSegs = totalSegs;
    P.colBlocks = (maxW + 255) / 256;
    const unsigned long long* dsb = ws.d_dsBase;
    const dim3 blk(kThreads);
    const int rowBlocks = (totalRows + 7) / 8;
    const int dsBlocks = (int)((ds + kThreads - 1) / kThreads);
    cudaEvent_t* tev = nullptr;
    if (ws.tevTicks > 0) {
        tev = &ws.tev[(size_t)ws.tevNext * (kTimedKernels + 1)];
        ws.tevNext = (ws.tevNext + 1) % ws.tevTicks;
        ws.tevRecorded = std::min(ws.tevRecorded + 1, ws.tevTicks);
    }
#define LV_TMARK(i) \
    if (tev) cudaEventRecord(tev[i], st)
    LV_TMARK(0);
    lvbgs_k_eval<<<totalTiles, blk, 0, st>>>(P);
    LV_TMARK(1);
    {
        // long scans: a grid sized to the device, striding over the list the evaluation built
        const int longBlocks = std::max(1, std::min(g_sm_count * 8, (int)((totalPx + kThreads - 1) / kThreads)));
        lvbgs_k_longscan<<<longBlocks, blk, 0, st>>>(P);
        LV_TMARK(2);
    }
    lvbgs_k_resolve<<<(totalTiles + kResolveTiles - 1) / kResolveTiles + dsBlocks, blk, 0, st>>>(P, ds, dsb);
    LV_TMARK(3);
    {
        const int grid = std::max(1, std::min(maxBlocks / std::max(1, ws.repairDiv), std::max(1, totalTiles)));
        void* args[] = {&P};
        LV_CUDA(errh, cudaLaunchCooperativeKernel((const void*)lvbgs_k_repair, dim3(grid), blk, args, 0, st),
                "repair kernel launch");
    }
    LV_TMARK(4);
    lvbgs_k_commit<<<totalTiles, blk, 0, st>>>(P);
    LV_TMARK(5);
    lvbgs_k_runs<<<rowBlocks, blk, 0, st>>>(P);
    LV_TMARK(6);
    lvbgs_k_vunion<<<rowBlocks, blk, 0, st>>>(P);
    LV_TMARK(7);
    lvbgs_k_holes<<<rowBlocks, blk, 0, st>>>(P);
    LV_TMARK(8);
    lvbgs_k_combine<<<rowBlocks, blk, 0, st>>>(P);
    LV_TMARK(9);
    lvbgs_k_hcount<<<totalRows, 128, 0, st>>>(P);
    LV_TMARK(10);
    lvbgs_k_median<<<dim3(P.colBlocks, std::max(1, totalSegs)), blk, 0, st>>>(P);
    LV_TMARK(11);
    lvbgs_k_epilogue<<<1, 128, 0, st>>>(P);
    LV_TMARK(12);
    lvbgs_k_dilate<<<totalRows, 128, 0, st>>>(P);
    LV_TMARK(13);
    lvbgs_k_reset<<<std::max(1, std::min(totalTiles, g_sm_count * 8)), blk, 0, st>>>(P);
    LV_TMARK(14);
    lvbgs_k_close<<<1, 128, 0, st>>>(P);
    LV_TMARK(15);
#undef LV_TMARK
    LV_CUDA(errh, cudaGetLastError(), "frame step launch");
    return LVBGS_OK;
}
lvbgs_status launch_tick(lvbgs_handle errh, Workspace& ws, int n, cudaStream_t st) {
    ws.h_dsBase.resize(n + 1);
    return launch_tick(errh, ws, n, st, ws.h_streams.data(), ws.h_dsBase.data());
}

// the device-side error flags of a tick as a status
lvbgs_status status_from_work(lvbgs_handle errh, const TickWork& w) {
    if (w.err & ERR_BARRIER_TIMEOUT) return fail(errh, LVBGS_DEVICE_TIMEOUT, "grid barrier wait timed out");
    if (w.err & ERR_REPAIR_LIMIT) return fail(errh, LVBGS_DEVICE_ERROR, "raster-order repair did not converge");
    if (w.err & ERR_UF_LIMIT) return fail(errh, LVBGS_DEVICE_ERROR, "hole-filling union-find exceeded its bound");
    if (w.err & ERR_RING) return fail(errh, LVBGS_DEVICE_ERROR, "closed mask is not zero at pixel (0,0)");
    return LVBGS_OK;
}
lvbgs_status read_work_status(lvbgs_handle errh, Workspace& ws) {
    TickWork w;
    LV_CUDA(errh, cudaMemcpy(&w, ws.work, sizeof(TickWork), cudaMemcpyDeviceToHost), "status read-back");
    return status_from_work(errh, w);
}

// stages a frame for the kernel: returns the device pointer the kernel reads
lvbgs_status stage_frame(lvbgs_handle h, const uint8_t* img, size_t stride, cudaStream_t st, const uint8_t** out) {
    const size_t row = (size_t)h->W * h->C;
    if (stride == 0) stride = row;
    if (stride < row) return fail(h, LVBGS_BAD_ARG, "image stride is smaller than width*channels");
    const bool dev = is_device_ptr(img);
    if (dev && stride == row) {
        *out = img;
        return LVBGS_OK;
    }
    LV_CUDA(h,
            cudaMemcpy2DAsync(h->d_frame, row, img, stride, row, h->H, dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                              st),
            "frame upload");
    *out = h->d_frame;
    return LVBGS_OK;
}

void set_lr(StreamDev& S, double lr) {
    // nLearningRate of the BG branch (:277 / :421)
    if (std::isinf(lr)) {
        S.lrMode = 1;
        S.lrFixed = ~0ull;
    } else if (lr > 0) {
        S.lrMode = 1;
        S.lrFixed = (unsigned long long)std::ceil(lr);
    } else {
        S.lrMode = 0;
        S.lrFixed = 0;
    }
}

lvbgs_status check_ready(lvbgs_handle h) {
    if (!h) return fail(nullptr, LVBGS_BAD_ARG, "null handle");
    if (!h->initialized) return fail(h, LVBGS_NOT_INITIALIZED, "algo & model must be initialized first");
    if (h->spilled) return fail(h, LVBGS_NOT_INITIALIZED, "stream state is spilled to host memory; restore it first");
    if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    return LVBGS_OK;
}

// box max over a (2r+1)^2 window clipped to the image
void host_dilate(const std::vector<uint8_t>& src, std::vector<uint8_t>& dst, int W, int H, int r) {
    std::vector<uint8_t> tmp(src.size());
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            uint8_t v = 0;
            for (int d = -r; d <= r; ++d)
                if (x + d >= 0 && x + d < W) v = std::max(v, src[(size_t)y * W + x + d]);
            tmp[(size_t)y * W + x] = v;
        }
    dst.assign(src.size(), 0);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            uint8_t v = 0;
            for (int d = -r; d <= r; ++d)
                if (y + d >= 0 && y + d < H) v = std::max(v, tmp[(size_t)(y + d) * W + x]);
            dst[(size_t)y * W + x] = v;
        }
}

uint8_t sat_round_u8(float v) {
    const long r = std::lrint(v);
    return (uint8_t)(r < 0 ? 0 : r > 255 ? 255 : r);
}

}  // namespace

// library-level error message (lvbgs_last_error(NULL)) for entry points defined in other files
lvbgs_status lvbgs::report_error(lvbgs_status st, const char* msg) { return fail(nullptr, st, msg); }

extern "C" {

// ==========================================================================================
// PAWCS (one channel): device layout, initialization and the frame step
// ==========================================================================================
namespace {

enum {
    PL_CTL = 0, PL_PCTL, PL_FM, PL_WCOLOR, PL_WDESC, PL_WOCC, PL_WFIRST, PL_WLAST, PL_ILLUM, PL_UNST, PL_ROI,
    PL_BLINKS, PL_LASTRAWFG, PL_LASTFG, PL_DILINV, PL_LASTRAWBLINK, PL_LASTCOL, PL_LASTDESC, PL_KCTR, PL_GLUT,
    PL_GMAP, PL_DSLT, PL_DSST, PL_DSROI,
    // scratch (not part of the model)
    PL_BITS, PL_HCOUNT, PL_LABEL, PL_INTENT, PL_DESCT, PL_REC, PL_OUT, PL_REPB, PL_REPA, PL_UFINAL, PL_UV,
    PL_ITEMLIST, PL_CONTRIBLIST, PL_BLKCOUNTS, PL_CATINFO, PL_DSABS, PL_UPDLIST, PL_GITEM, PL_CONTRIB, PL_DSFRAME, PL_FRAME, PL_MASK, PL_ROWSUM, PL_WORK, PL_FLAGS, PL_PDEV, PL_SDEV, PL_DIRTY, PL_GSEG, PL_GCAND, PL_GTRUE, PL_COUNT
};
struct PwLayout {
    size_t off[PL_COUNT];
    size_t persist, total;
};
PwLayout pw_layout(int W, int H, int C, int L, int G) {
    const size_t npx = (size_t)W * H, gmap = (size_t)(W / 2) * (H / 2), nds = (size_t)(W / 8) * (H / 8);
    size_t sz[PL_COUNT];
    sz[PL_CTL] = sizeof(StreamCtl);
    sz[PL_PCTL] = sizeof(PawcsCtl);
    sz[PL_FM] = 2 * kNumFloatMaps * npx * 4;
    // word colours / descriptors: [2][L][npx] one channel, [2][L][npx][3] three (channel-minor)
    sz[PL_WCOLOR] = 2 * (size_t)L * npx * C;
    sz[PL_WDESC] = 2 * (size_t)L * npx * 2 * C;
    sz[PL_WOCC] = sz[PL_WFIRST] = sz[PL_WLAST] = 2 * (size_t)L * npx * 4;
    sz[PL_ILLUM] = sz[PL_UNST] = sz[PL_ROI] = sz[PL_BLINKS] = sz[PL_LASTRAWFG] = sz[PL_LASTFG] = sz[PL_DILINV] =
        sz[PL_LASTRAWBLINK] = npx;
    sz[PL_LASTCOL] = npx * C;
    sz[PL_LASTDESC] = npx * 2 * C;
    sz[PL_KCTR] = npx * 2;
    sz[PL_GLUT] = npx * kPwGlutStride;
    sz[PL_GMAP] = (size_t)G * std::max<size_t>(gmap, 1) * 4;
    sz[PL_DSLT] = sz[PL_DSST] = std::max<size_t>(nds, 1) * 4 * C;
    sz[PL_DSROI] = std::max<size_t>(nds, 1);
    sz[PL_BITS] = bit_planes_bytes(W, H);
    sz[PL_HCOUNT] = npx;
    sz[PL_LABEL] = sz[PL_INTENT] = npx * 4;
    sz[PL_DESCT] = npx * 2 * C;
    sz[PL_REC] = npx * sizeof(PwRec);
    sz[PL_OUT] = npx * sizeof(PwOut);
    sz[PL_REPB] = sz[PL_REPA] = npx * 4;
    sz[PL_UFINAL] = npx;
    sz[PL_UV] = npx;
    sz[PL_ITEMLIST] = npx * 32;
    sz[PL_CONTRIBLIST] = npx * 4;
    sz[PL_BLKCOUNTS] = ((npx + kPwCompactBlk - 1) / kPwCompactBlk) * kPwCats * 4;
    sz[PL_CATINFO] = 2 * kPwCatBase * 4;
    sz[PL_DSABS] = std::max<size_t>(nds, 1) * 4;
    sz[PL_UPDLIST] = npx * 4;
    sz[PL_GITEM] = npx * 4;
    sz[PL_CONTRIB] = npx * 4;
    sz[PL_DSFRAME] = std::max<size_t>(nds, 1) * C;
    sz[PL_FRAME] = npx * C;
    sz[PL_MASK] = npx;
    sz[PL_ROWSUM] = (size_t)kPwMaxGlobal * std::max<size_t>(gmap, 1) * 8;
    sz[PL_WORK] = sizeof(TickWork);
    sz[PL_FLAGS] = 64;
    sz[PL_PDEV] = sizeof(PawcsDev);
    sz[PL_SDEV] = sizeof(StreamDev);
    sz[PL_DIRTY] = npx;
    sz[PL_GSEG] = (npx / 512 + 2) * 24 * 4;
    sz[PL_GCAND] = npx * 4;
    sz[PL_GTRUE] = npx;
    PwLayout Lo;
    size_t o = 0;
    for (int i = 0; i < PL_COUNT; ++i) {
        if (i == PL_BITS) Lo.persist = o;
        Lo.off[i] = o;
        o += align256(sz[i]);
    }
    Lo.total = o;
    return Lo;
}

// resolution-dependent parameters of BackgroundSubtractorPAWCS::initialize (:446-466)
struct PwGeom {
    int L, G, median_k, big;
};
PwGeom pw_geometry(const lvbgs_params& prm, size_t npx, size_t orig, int C) {
    PwGeom g;
    size_t L = prm.bg_samples, maxG = prm.bg_samples / 2, G;
    const int k = prm.default_median_blur_kernel_size;
    int raw;
    if (orig >= npx / 2 && (int)npx >= 320 * 240) {
        const float f = (float)npx / (320 * 240);
        raw = std::min((int)std::floor(0.5f + f) + k, k + 4);
        G = maxG;
        g.big = 1;
    } else {
        const float f = (float)orig / (320 * 240);
        raw = std::min((int)std::floor(0.5f + (float)k * f * 2) + (k - 4), k);
        const size_t gg = (size_t)std::pow((double)((float)maxG * f), 2) + 1;
        G = std::min(gg, maxG);
        g.big = 0;
    }
    g.median_k = (raw % 2) ? raw : raw - 1;
    if (C == 1) {
        L = std::max<size_t>(L / 2, 1);
        G = std::max<size_t>(G / 2, 1);
    }
    g.L = (int)L;
    g.G = (int)G;
    return g;
}

void pw_fill(lvbgs_ctx* h, const PwLayout& Lo, int L, int G) {
    uint8_t* b = h->dmem;
    StreamDev& S = h->sd;
    std::memset(&S, 0, sizeof(S));
    S.ctl = (StreamCtl*)(b + Lo.off[PL_CTL]);
    S.fm = (float*)(b + Lo.off[PL_FM]);
    S.roi = b + Lo.off[PL_ROI];
    S.blinks = b + Lo.off[PL_BLINKS];
    S.lastRawFG = b + Lo.off[PL_LASTRAWFG];
    S.lastFG = b + Lo.off[PL_LASTFG];
    S.dilInv = b + Lo.off[PL_DILINV];
    S.lastRawBlink = b + Lo.off[PL_LASTRAWBLINK];
    S.lastCol = b + Lo.off[PL_LASTCOL];
    S.lastDesc = (uint16_t*)(b + Lo.off[PL_LASTDESC]);
    S.kctr = (uint16_t*)(b + Lo.off[PL_KCTR]);
    S.dsLT = (float*)(b + Lo.off[PL_DSLT]);
    S.dsST = (float*)(b + Lo.off[PL_DSST]);
    S.bits = (uint32_t*)(b + Lo.off[PL_BITS]);
    S.hcount = b + Lo.off[PL_HCOUNT];
    S.label = (int*)(b + Lo.off[PL_LABEL]);
    S.intent = (uint32_t*)(b + Lo.off[PL_INTENT]);
    h->d_frame = b + Lo.off[PL_FRAME];
    h->d_mask = b + Lo.off[PL_MASK];
    fill_geometry(h);
    PawcsDev& D = h->pd;
    D.pc = (PawcsCtl*)(b + Lo.off[PL_PCTL]);
    D.L = L;
    D.G = G;
    D.gwW = h->W / 2;
    D.gwH = h->H / 2;
    D.minColor = (unsigned)h->prm.min_color_dist_threshold;
    D.descOff = (unsigned)h->prm.desc_dist_threshold_offset;
    D.nmv = (unsigned)h->prm.samples_for_moving_avgs;
    D.relThr = h->prm.rel_lbsp_threshold;
    D.lbspOff = (unsigned)h->prm.lbsp_threshold_offset;
    D.wColor = b + Lo.off[PL_WCOLOR];
    D.wDesc = (uint16_t*)(b + Lo.off[PL_WDESC]);
    D.wOcc = (uint32_t*)(b + Lo.off[PL_WOCC]);
    D.wFirst = (uint32_t*)(b + Lo.off[PL_WFIRST]);
    D.wLast = (uint32_t*)(b + Lo.off[PL_WLAST]);
    D.illum = b + Lo.off[PL_ILLUM];
    D.unstable = b + Lo.off[PL_UNST];
    D.glut = b + Lo.off[PL_GLUT];
    D.gmap = (float*)(b + Lo.off[PL_GMAP]);
    D.descT = (uint16_t*)(b + Lo.off[PL_DESCT]);
    D.rec = (PwRec*)(b + Lo.off[PL_REC]);
    D.out = (PwOut*)(b + Lo.off[PL_OUT]);
    D.repBefore = (uint32_t*)(b + Lo.off[PL_REPB]);
    D.repAfter = (uint32_t*)(b + Lo.off[PL_REPA]);
    D.uFinal = b + Lo.off[PL_UFINAL];
    D.uv = b + Lo.off[PL_UV];
    D.itemList = (uint4*)(b + Lo.off[PL_ITEMLIST]);
    D.contribList = (float*)(b + Lo.off[PL_CONTRIBLIST]);
    D.blkCounts = (uint32_t*)(b + Lo.off[PL_BLKCOUNTS]);
    D.catInfo = (uint32_t*)(b + Lo.off[PL_CATINFO]);
    D.dsAbs = (float*)(b + Lo.off[PL_DSABS]);
    D.updList = (uint32_t*)(b + Lo.off[PL_UPDLIST]);
    D.gitem = (uint32_t*)(b + Lo.off[PL_GITEM]);
    D.contrib = (float*)(b + Lo.off[PL_CONTRIB]);
    D.dsRoi = b + Lo.off[PL_DSROI];
    D.dsFrame = b + Lo.off[PL_DSFRAME];
    D.dirty = b + Lo.off[PL_DIRTY];
    D.gseg = (uint32_t*)(b + Lo.off[PL_GSEG]);
    D.gcand = (uint32_t*)(b + Lo.off[PL_GCAND]);
    D.gtrue = b + Lo.off[PL_GTRUE];
    h->d_rowsum = (double*)(b + Lo.off[PL_ROWSUM]);
    h->d_work = (TickWork*)(b + Lo.off[PL_WORK]);
    h->d_flags = (unsigned int*)(b + Lo.off[PL_FLAGS]);
    h->d_pd = (PawcsDev*)(b + Lo.off[PL_PDEV]);
    h->d_sd = (StreamDev*)(b + Lo.off[PL_SDEV]);
}

PwParams pw_params(lvbgs_ctx* h, double lr) {
    PwParams P;
    P.streams = h->d_pd;
    P.nStreams = 1;
    P.totalTiles = h->sd.nTiles;
    P.totalRows = h->H;
    P.totalCells = h->pd.gwW * h->pd.gwH;
    P.round = 0;
    P.lr = lr;
    P.flags = h->d_flags;
    P.conv = nullptr;
    return P;
}

lvbgs_status pw_upload_desc(lvbgs_ctx* h, cudaStream_t st) {
    h->pd.sd = h->sd;
    LV_CUDA(h, cudaMemcpyAsync(h->d_pd, &h->pd, sizeof(PawcsDev), cudaMemcpyHostToDevice, st), "descriptor upload");
    LV_CUDA(h, cudaMemcpyAsync(h->d_sd, &h->sd, sizeof(StreamDev), cudaMemcpyHostToDevice, st), "descriptor upload");
    return LVBGS_OK;
}

// refreshModel(nBaseOccCount, fOccDecrFrac, bForceFGUpdate) of the dictionaries in buffer buf at frame t
lvbgs_status pw_refresh(lvbgs_ctx* h, uint32_t t, int buf, int baseOcc, float decr, int force, int onlyPending,
                        int useDil, cudaStream_t st) {
    const int npx = (int)h->npx;
    if (h->C == 3) {
        pw3_k_refresh_local<<<(npx + 127) / 128, 128, 0, st>>>(h->pd, t, buf, baseOcc, decr, force, onlyPending, useDil);
        pw3_k_refresh_global<<<1, 1, 0, st>>>(h->pd, t, buf, force, onlyPending, useDil);
    } else {
        pw_k_refresh_local<<<(npx + 127) / 128, 128, 0, st>>>(h->pd, t, buf, baseOcc, decr, force, onlyPending, useDil);
        pw_k_refresh_global<<<1, 1, 0, st>>>(h->pd, t, buf, force, onlyPending, useDil);
    }
    PwParams P = pw_params(h, 0.0);
    pw_k_lut_sort<<<h->sd.nTiles, kThreads, 0, st>>>(P, onlyPending ? 2 : 1);
    LV_CUDA(h, cudaGetLastError(), "refresh kernel launch");
    return LVBGS_OK;
}

lvbgs_status pw_initialize(lvbgs_ctx* h, const uint8_t* img, int W, int H, int C, size_t stride,
                           const std::vector<uint8_t>& newroi, size_t orig, size_t fin) {
    if (C != 1 && C != 3) return fail(h, LVBGS_UNSUPPORTED, "PAWCS runs on single- and three-channel frames");
    const size_t npx = (size_t)W * H;
    const PwGeom g = pw_geometry(h->prm, npx, orig, C);
    if (g.L > (C == 3 ? kPw3MaxLocal : kPwMaxLocal) || g.G > kPwMaxGlobal)
        return fail(h, LVBGS_UNSUPPORTED, "word counts above the supported maximum");
    if (g.median_k > 13) return fail(h, LVBGS_UNSUPPORTED, "median kernel sizes above 13 are not supported");
    const int dsW = W / 8, dsH = H / 8;
    // the reference's cv::resize to (W/8, H/8) (:446) needs a non-empty output
    if (dsW <= 0 || dsH <= 0) return fail(h, LVBGS_BAD_SIZE, "frames must be at least 8x8 pixels");
    // down-sampled ROI (INTER_AREA of the validated ROI, :446) and its pixel count
    std::vector<uint8_t> dsRoi((size_t)dsW * dsH);
    size_t dsCount = 0;
    for (int y = 0; y < dsH; ++y)
        for (int x = 0; x < dsW; ++x) {
            uint8_t v = area_resample(W, H, dsW, dsH, x, y, [&](int sx, int sy) { return (int)newroi[(size_t)sy * W + sx]; });
            if (g.big) v |= 127;
            dsRoi[(size_t)y * dsW + x] = v;
            dsCount += v != 0;
        }
    StreamCtl ctl;
    std::memset(&ctl, 0, sizeof(ctl));
    ctl.auto_reset = 1;  // IIBackgroundSubtractor's default (BackgroundSubtractionUtils.cpp:67)
    ctl.median_k = g.median_k;
    const float rel = h->prm.rel_lbsp_threshold;
    // BackgroundSubtractorLBSP.cpp:30-34: one channel divides the threshold by 3
    for (int t = 0; t <= 255; ++t)
        ctl.lut[t] = C == 1 ? sat_round_u8(((float)t * rel + (float)h->prm.lbsp_threshold_offset) / 3)
                            : sat_round_u8((float)t * rel + (float)h->prm.lbsp_threshold_offset);
    ctl.n_rel = fin;
    ctl.orig_roi = orig;
    {
        // factors of frame 1 (bootstrapping: N/2 and N/8 frames)
        const unsigned long long nlt = h->prm.samples_for_moving_avgs / 2, nst = nlt / 4;
        ctl.fLT = 1.0f / (float)(1ull < nlt ? 1ull : nlt);
        ctl.fST = 1.0f / (float)(1ull < nst ? 1ull : nst);
        ctl.bLT = (float)((1.0 / 255) * (double)ctl.fLT);
        ctl.bST = (float)((1.0 / 255) * (double)ctl.fST);
    }
    PawcsCtl pc;
    std::memset(&pc, 0, sizeof(pc));
    pc.lword_offset = 1000;
    pc.L = g.L;
    pc.G = g.G;
    pc.ds_roi_count = dsCount;
    for (int i = 0; i < kPwMaxGlobal; ++i) pc.gdict[i] = -1;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->dmem);
    h->dmem = nullptr;
    h->initialized = false;
    h->spilled = false;
    const PwLayout Lo = pw_layout(W, H, C, g.L, g.G);
    LV_CUDA(h, cudaMalloc(&h->dmem, Lo.total), "model allocation");
    if (!h->h_flags) LV_CUDA(h, cudaHostAlloc((void**)&h->h_flags, 64, cudaHostAllocDefault), "pinned allocation");
    h->persistBytes = Lo.persist;
    h->totalBytes = Lo.total;
    h->W = W;
    h->H = H;
    h->C = C;
    h->npx = npx;
    h->roi = newroi;
    h->roiW = W;
    h->roiH = H;
    h->n_rel = fin;
    h->orig_roi = orig;
    h->pw_frames = 0;
    h->pw_offset = 1000;
    pw_fill(h, Lo, g.L, g.G);
    cudaStream_t st = h->stream;
    LV_CUDA(h, cudaMemsetAsync(h->dmem, 0, Lo.total, st), "model reset");
    LV_CUDA(h, cudaMemcpyAsync(h->sd.ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, st), "control upload");
    LV_CUDA(h, cudaMemcpyAsync(h->pd.pc, &pc, sizeof(pc), cudaMemcpyHostToDevice, st), "control upload");
    LV_CUDA(h, cudaMemcpyAsync(h->sd.roi, h->roi.data(), npx, cudaMemcpyHostToDevice, st), "roi upload");
    LV_CUDA(h, cudaMemcpyAsync(h->pd.dsRoi, dsRoi.data(), dsRoi.size(), cudaMemcpyHostToDevice, st), "roi upload");
    const uint8_t* dimg = nullptr;
    lvbgs_status s = stage_frame(h, img, stride, st, &dimg);
    if (s != LVBGS_OK) return s;
    if ((s = pw_upload_desc(h, st)) != LVBGS_OK) return s;
    if (C == 3) {
        pw3_k_init<<<1024, 256, 0, st>>>(h->pd);
        pw3_k_init_last<<<1024, 256, 0, st>>>(h->pd, dimg);
    } else {
        pw_k_init<<<1024, 256, 0, st>>>(h->pd);
        pw_k_init_last<<<1024, 256, 0, st>>>(h->pd, dimg);
    }
    LV_CUDA(h, cudaGetLastError(), "init kernel launch");
    // refreshModel(1, 0) at frame 0 (:555)
    if ((s = pw_refresh(h, 0u, 0, 1, 0.0f, 0, 0, 0, st)) != LVBGS_OK) return s;
    LV_CUDA(h, cudaStreamSynchronize(st), "initialization");
    h->initialized = true;
    return LVBGS_OK;
}

// LOBSTER initialize() (BackgroundSubtractorLOBSTER.cpp:442-457) on the validated ROI, or ViBe's
// (BackgroundSubtractorViBe.cpp:57-75 / :112-134) or PBAS's (BackgroundSubtractorPBAS.cpp:61-109 /
// :287-324) on every pixel
lvbgs_status lob_initialize(lvbgs_ctx* h, const uint8_t* img, int W, int H, int C, size_t stride,
                            const std::vector<uint8_t>& newroi, size_t orig, size_t fin) {
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->dmem);
    h->dmem = nullptr;
    h->initialized = false;
    h->spilled = false;
    std::string err;
    const int alg = h->algo == LVBGS_ALGO_VIBE ? ALG_VIBE : h->algo == LVBGS_ALGO_PBAS ? ALG_PBAS : ALG_LOBSTER;
    lvbgs_status s = lob_setup(*h->lob, alg, h->prm, W, H, C, newroi, orig, fin, h->stream, err);
    if (s != LVBGS_OK) return fail(h, s, err);
    h->W = W;
    h->H = H;
    h->C = C;
    h->npx = (size_t)W * H;
    h->roi = newroi;
    h->roiW = W;
    h->roiH = H;
    h->n_rel = fin;
    h->orig_roi = orig;
    h->d_frame = h->lob->d_frame;
    h->d_mask = h->lob->d_mask;
    h->persistBytes = h->totalBytes = h->lob->bytes;
    const uint8_t* dimg = nullptr;
    if ((s = stage_frame(h, img, stride, h->stream, &dimg)) != LVBGS_OK) return s;
    if ((s = lob_init_model(*h->lob, dimg, h->stream, err)) != LVBGS_OK) return fail(h, s, err);
    h->initialized = true;
    return LVBGS_OK;
}

// PAWCS frame steps are resumable: pw_begin enqueues a frame's first batch of fixed-point rounds and
// returns; pw_advance waits for the step's latest read-back and enqueues what follows (more rounds, the
// camera-motion decision, the rest of the frame), until the step is done. lvbgs_apply runs one step to
// the end; a batch keeps the steps of several PAWCS streams in flight on their own CUDA streams.
double pw_ms_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ordered compaction: mode 0 lists the critical global items, mode 1 the word weight contributions,
// mode 2 the neighbour-update loops
void pw_compact(lvbgs_ctx* h, const PwParams& Pc, int mode, cudaStream_t st) {
    const int cblocks = (int)((h->npx + kPwCompactBlk - 1) / kPwCompactBlk);
    pw_k_compact_count<<<cblocks, 256, 0, st>>>(Pc, mode);
    const int ncat = mode == 1 ? h->pd.G : 1;
    pw_k_compact_offsets<<<1, 32 * std::min(ncat, 32), 0, st>>>(Pc, ncat);
    pw_k_compact_scatter<<<cblocks, 256, 0, st>>>(Pc, mode);
}

// enqueues fixed-point rounds enq .. enq+n-1 (each ends with pw_k_round_end; once a round finds no dirty
// pixel every later kernel of the rounds returns at once, PW_ROUND_GUARD) and the read-back of the
// converged flag and round count
lvbgs_status pw_enqueue_rounds(lvbgs_ctx* h, int n) {
    PwStep& w = h->pws;
    const cudaStream_t st = w.st;
    const dim3 blk(kThreads);
    const int tiles = h->sd.nTiles;
    const int cblocks = (int)((h->npx + kPwCompactBlk - 1) / kPwCompactBlk);
    for (int r = 0; r < n && w.enq < w.maxRounds; ++r, ++w.enq) {
        w.PR.round = w.enq;
        const PwParams& P = w.PR;
        if (h->C == 3) {
            // three channels: the local pass applies the earlier updaters' loops itself
            pw3_k_local<<<tiles, blk, 0, st>>>(P);
            pw_k_illum<<<(h->H + 7) / 8, 256, 0, st>>>(P);
            pw_compact(h, P, 0, st);
            pw3_k_gscan_seg<<<(int)((h->npx + 4 * 512 - 1) / (4 * 512)), 128, 0, st>>>(P);
            pw3_k_gscan_walk<<<1, 32, 0, st>>>(P);
            pw3_k_gscan_fix<<<(int)((h->npx + 255) / 256), 256, 0, st>>>(P);
            pw3_k_gscan_fix_walked<<<(int)((h->npx + 4 * 512 - 1) / (4 * 512)), 128, 0, st>>>(P);
            pw_k_cells<<<(P.totalCells + 255) / 256, 256, 0, st>>>(P, 0);
            pw_k_nbr<<<tiles, blk, 0, st>>>(P);
            LV_CUDA(h, cudaMemsetAsync(h->d_flags, 0, 4, st), "flag reset");
            pw3_k_dirty<<<tiles, blk, 0, st>>>(P);
        } else {
            pw_k_local<<<tiles, blk, 0, st>>>(P);
            pw_k_illum<<<(h->H + 7) / 8, 256, 0, st>>>(P);
            pw_compact(h, P, 0, st);
            pw3_k_gscan_seg<<<(int)((h->npx + 4 * 512 - 1) / (4 * 512)), 128, 0, st>>>(P);
            pw3_k_gscan_walk<<<1, 32, 0, st>>>(P);
            pw3_k_gscan_fix<<<(int)((h->npx + 255) / 256), 256, 0, st>>>(P);
            pw3_k_gscan_fix_walked<<<(int)((h->npx + 4 * 512 - 1) / (4 * 512)), 128, 0, st>>>(P);
            pw_k_cells<<<(P.totalCells + 255) / 256, 256, 0, st>>>(P, 0);
            pw_k_nbr<<<tiles, blk, 0, st>>>(P);
            pw_compact(h, P, 2, st);
            pw_k_nbr_loops<<<std::max(1, std::min(cblocks * 4, 1216)), 256, 0, st>>>(P);
            pw_k_replace<<<tiles, blk, 0, st>>>(P);
            LV_CUDA(h, cudaMemsetAsync(h->d_flags, 0, 4, st), "flag reset");
            pw_k_dirty<<<tiles, blk, 0, st>>>(P);
        }
        pw_k_round_end<<<1, 1, 0, st>>>(P);
    }
    LV_CUDA(h, cudaGetLastError(), "PAWCS round launch");
    LV_CUDA(h, cudaMemcpyAsync(h->h_flags + 3, h->d_flags + 3, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, st),
            "flag read-back");
    return LVBGS_OK;
}

// one PAWCS frame step: local passes to the raster-order fixed point (enqueued ahead, as many rounds as
// the previous frame needed, then one at a time), then commit, global words, post-processing and the
// frame level. Host time of the parts goes to pw_host_ms (lvbgs_debug_pawcs_host_timing).
lvbgs_status pw_begin(lvbgs_ctx* h, const uint8_t* img, size_t stride, uint8_t* mask, double lr, cudaStream_t st) {
    const std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    for (double& v : h->pw_host_ms) v = 0.0;
    PwStep& w = h->pws;
    w = PwStep();
    w.st = st;
    const uint8_t* dimg = nullptr;
    lvbgs_status s = stage_frame(h, img, stride, st, &dimg);
    if (s != LVBGS_OK) return s;
    w.mask = mask;
    w.devMask = mask_writable_by_device(mask);
    h->sd.frame = dimg;
    h->sd.maskOut = w.devMask ? mask : h->d_mask;
    if ((s = pw_upload_desc(h, st)) != LVBGS_OK) return s;
    w.P = pw_params(h, lr);
    LV_CUDA(h, cudaMemsetAsync(h->pd.repBefore, 0xff, h->npx * 4, st), "scratch reset");
    LV_CUDA(h, cudaMemsetAsync(h->d_work, 0, sizeof(TickWork), st), "scratch reset");
    w.maxRounds = h->dbg_fault == LVBGS_FAULT_PAWCS_ROUNDS ? 1 : 64;
    h->dbg_fault = 0;
    LV_CUDA(h, cudaMemsetAsync(h->d_flags, 0, 5 * sizeof(unsigned int), st), "flag reset");
    w.PR = w.P;
    w.PR.conv = h->d_flags + 3;
    w.enq = 0;
    s = pw_enqueue_rounds(h, std::max(1, std::min(h->pw_rounds_last, w.maxRounds)));
    w.stage = 0;
    w.active = s == LVBGS_OK;
    h->pw_host_ms[0] += pw_ms_since(t0);
    return s;
}

// the rest of the frame after the fixed point, up to the camera-motion decision (enqueued with its
// read-back on frames that take it: returns true) or to the end (returns false)
lvbgs_status pw_enqueue_tail_a(lvbgs_ctx* h, bool& motion) {
    PwStep& w = h->pws;
    const cudaStream_t st = w.st;
    const PwParams& P = w.P;
    const dim3 blk(kThreads);
    const int tiles = h->sd.nTiles;
    const bool c3 = h->C == 3;
    if (c3) {
        pw3_k_later<<<tiles, blk, 0, st>>>(P);
        pw3_k_commit<<<tiles, blk, 0, st>>>(P);
    } else {
        pw_k_commit<<<tiles, blk, 0, st>>>(P);
    }
    pw_k_cells<<<(P.totalCells + 255) / 256, 256, 0, st>>>(P, 1);
    pw_compact(h, P, 1, st);
    pw_k_weights<<<kPwMaxGlobal, 256, 0, st>>>(P);
    pw_k_gw_recalc<<<kPwMaxGlobal, 256, 0, st>>>(P);
    pw_k_gw_decay<<<dim3(64, kPwMaxGlobal), 256, 0, st>>>(P, h->d_rowsum);
    pw_k_gw_blur<<<dim3(64, kPwMaxGlobal), 256, 0, st>>>(P, h->d_rowsum);
    pw_k_gw_sort<<<1, 32, 0, st>>>(P);
    pw_k_lut_sort<<<tiles, blk, 0, st>>>(P, 0);
    pw_k_blink_close<<<tiles, blk, 0, st>>>(P);
    TickParams TP;
    std::memset(&TP, 0, sizeof(TP));
    TP.streams = h->d_sd;
    TP.nStreams = 1;
    TP.totalTiles = tiles;
    TP.totalRows = h->H;
    TP.work = h->d_work;
    TP.totalSegs = h->sd.nSegs;
    TP.colBlocks = (h->W + 255) / 256;
    const int rowBlocks = (h->H + 7) / 8;
    lvbgs_k_runs<<<rowBlocks, blk, 0, st>>>(TP);
    lvbgs_k_vunion<<<rowBlocks, blk, 0, st>>>(TP);
    lvbgs_k_holes<<<rowBlocks, blk, 0, st>>>(TP);
    lvbgs_k_combine<<<rowBlocks, blk, 0, st>>>(TP);
    lvbgs_k_hcount<<<h->H, 128, 0, st>>>(TP);
    lvbgs_k_median<<<dim3(TP.colBlocks, TP.totalSegs), blk, 0, st>>>(TP);
    lvbgs_k_dilate<<<h->H, 128, 0, st>>>(TP);
    const int nds = (h->W / 8) * (h->H / 8);
    if (nds > 0) {
        if (c3) pw3_k_ds<<<(nds + 255) / 256, 256, 0, st>>>(P);
        else pw_k_ds<<<(nds + 255) / 256, 256, 0, st>>>(P);
    }
    pw_k_epilogue<<<1, 256, 0, st>>>(P);
    const uint32_t t = (uint32_t)(h->pw_frames + 1);
    motion = nds > 0 && t % kPwBootWin == 0;
    if (motion) {
        // camera-motion comparison (:1480-1501): the host waits for the decision, which may switch the
        // local word weight offset and run refreshModel(1, 1, true)
        const int nxt = (int)((h->pw_frames & 1ull) ^ 1ull);
        if (c3) pw3_k_motion_bg<<<(nds + 255) / 256, 256, 0, st>>>(P, nxt);
        else pw_k_motion_bg<<<(nds + 255) / 256, 256, 0, st>>>(P, nxt);
        pw_k_motion_decide<<<1, 32, 0, st>>>(P);
        LV_CUDA(h, cudaGetLastError(), "PAWCS camera-motion launch");
        LV_CUDA(h, cudaMemcpyAsync(h->h_flags + 1, h->d_flags + 1, 8, cudaMemcpyDeviceToHost, st), "flag read-back");
    }
    return LVBGS_OK;
}

// the end of the frame: the automatic model reset and the mask download
lvbgs_status pw_enqueue_tail_b(lvbgs_ctx* h) {
    PwStep& w = h->pws;
    const cudaStream_t st = w.st;
    const PwParams& P = w.P;
    const uint32_t t = (uint32_t)(h->pw_frames + 1);
    const int nxt = (int)((h->pw_frames & 1ull) ^ 1ull);
    pw_k_reset_decide<<<1, 32, 0, st>>>(P);
    // automatic model reset (:1503-1508): refreshModel(offset/8, 0, true) and T(x) := 1
    lvbgs_status s = pw_refresh(h, t, nxt, (int)(h->pw_offset / 8), 0.0f, 1, 1, 1, st);
    if (s != LVBGS_OK) return s;
    pw_k_reset_T<<<256, 256, 0, st>>>(h->pd, nxt);
    pw_k_close<<<1, 32, 0, st>>>(P);
    LV_CUDA(h, cudaGetLastError(), "PAWCS frame step launch");
    if (w.mask && !w.devMask)
        LV_CUDA(h, cudaMemcpyAsync(w.mask, h->d_mask, h->npx, cudaMemcpyDeviceToHost, st), "mask download");
    return LVBGS_OK;
}

// waits for the step's latest read-back and enqueues what follows; done is set when the step is over
lvbgs_status pw_advance(lvbgs_ctx* h, bool& done) {
    PwStep& w = h->pws;
    done = false;
    if (!w.active) {
        done = true;
        return fail(h, LVBGS_BAD_ARG, "no PAWCS frame step in flight");
    }
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    auto finish = [&](lvbgs_status s) {
        w.active = false;
        done = true;
        return s;
    };
    cudaError_t e = cudaStreamSynchronize(w.st);
    h->pw_host_ms[w.stage == 0 ? 1 : w.stage == 1 ? 2 : 3] += pw_ms_since(t0);
    if (e != cudaSuccess) return finish(cuda_fail(h, e, w.stage == 0 ? "PAWCS rounds" : "PAWCS frame step"));
    t0 = std::chrono::steady_clock::now();
    lvbgs_status s = LVBGS_OK;
    if (w.stage == 0) {
        if (!h->h_flags[3]) {
            if (w.enq >= w.maxRounds)
                return finish(fail(h, LVBGS_DEVICE_ERROR, "PAWCS raster-order fixed point did not converge in the round limit"));
            s = pw_enqueue_rounds(h, 1);
            h->pw_host_ms[0] += pw_ms_since(t0);
            return s == LVBGS_OK ? s : finish(s);
        }
        h->pw_rounds_last = (int)h->h_flags[4];
        bool motion = false;
        if ((s = pw_enqueue_tail_a(h, motion)) != LVBGS_OK) return finish(s);
        if (motion) {
            w.stage = 1;
            h->pw_host_ms[2] += pw_ms_since(t0);
            return LVBGS_OK;
        }
        s = pw_enqueue_tail_b(h);
        w.stage = 2;
        h->pw_host_ms[2] += pw_ms_since(t0);
        return s == LVBGS_OK ? s : finish(s);
    }
    if (w.stage == 1) {
        if (h->h_flags[1]) {
            h->pw_offset = h->h_flags[2];
            const uint32_t t = (uint32_t)(h->pw_frames + 1);
            const int nxt = (int)((h->pw_frames & 1ull) ^ 1ull);
            if ((s = pw_refresh(h, t, nxt, 1, 1.0f, 1, 0, 1, w.st)) != LVBGS_OK) return finish(s);
        }
        s = pw_enqueue_tail_b(h);
        w.stage = 2;
        h->pw_host_ms[2] += pw_ms_since(t0);
        return s == LVBGS_OK ? s : finish(s);
    }
    // stage 2: the frame step is over
    h->pw_frames += 1;
    TickWork tw;
    e = cudaMemcpy(&tw, h->d_work, sizeof(TickWork), cudaMemcpyDeviceToHost);
    h->pw_host_ms[4] += pw_ms_since(t0);
    if (e != cudaSuccess) return finish(cuda_fail(h, e, "status read-back"));
    return finish(status_from_work(h, tw));
}

lvbgs_status pw_apply(lvbgs_ctx* h, const uint8_t* img, size_t stride, uint8_t* mask, double lr, cudaStream_t st) {
    lvbgs_status s = pw_begin(h, img, stride, mask, lr, st);
    if (s != LVBGS_OK) {
        h->pws.active = false;
        return s;
    }
    bool done = false;
    while (!done) s = pw_advance(h, done);
    return s;
}

}  // namespace

lvbgs_status lvbgs_debug_pawcs_host_timing(lvbgs_handle h, double* out_ms) {
    if (!h || !out_ms) return fail(nullptr, LVBGS_BAD_ARG, "null argument");
    if (h->algo != LVBGS_ALGO_PAWCS) return fail(h, LVBGS_BAD_ARG, "not a PAWCS handle");
    for (int i = 0; i < 5; ++i) out_ms[i] = h->pw_host_ms[i];
    return LVBGS_OK;
}

lvbgs_status lvbgs_debug_inject_fault(lvbgs_handle h, int kind) {
    if (!h) return fail(nullptr, LVBGS_BAD_ARG, "null handle");
    if (kind < LVBGS_FAULT_NONE || kind > LVBGS_FAULT_PAWCS_ROUNDS) return fail(h, LVBGS_BAD_ARG, "unknown fault kind");
    h->dbg_fault = kind;
    return LVBGS_OK;
}

lvbgs_status lvbgs_default_params(lvbgs_algo algo, lvbgs_params* out) {
    if (!out) return fail(nullptr, LVBGS_BAD_ARG, "null output");
    out->update_rate = 16.0f;  // PBAS's BGSPBAS_DEFAULT_LEARNING_RATE (BackgroundSubtractorPBAS.hpp:55)
    if (algo == LVBGS_ALGO_PBAS) {
        // BackgroundSubtractorPBAS.hpp:48-55 (min_color_dist_threshold carries nInitColorDistThreshold)
        out->desc_dist_threshold_offset = 0;
        out->min_color_dist_threshold = 30;
        out->bg_samples = 35;
        out->required_bg_samples = 2;
        out->samples_for_moving_avgs = 100;
        out->rel_lbsp_threshold = 0.333f;
        out->lbsp_threshold_offset = 0;
        out->default_median_blur_kernel_size = 9;
        out->seed = 0;
        out->device_id = 0;
        return LVBGS_OK;
    }
    if (algo == LVBGS_ALGO_PAWCS) {
        // BackgroundSubtractorPAWCS.hpp:22-29 (bg_samples carries nMaxNbWords), BackgroundSubtractorLBSP.hpp:23-28
        out->desc_dist_threshold_offset = 2;
        out->min_color_dist_threshold = 20;
        out->bg_samples = 50;
        out->required_bg_samples = 0;
        out->samples_for_moving_avgs = 100;
        out->rel_lbsp_threshold = 0.333f;
        out->lbsp_threshold_offset = 0;
        out->default_median_blur_kernel_size = 9;
        out->seed = 0;
        out->device_id = 0;
        return LVBGS_OK;
    }
    if (algo == LVBGS_ALGO_LOBSTER) {
        // BackgroundSubtractorLOBSTER.hpp:22-31 (desc_dist_threshold_offset carries nDescDistThreshold,
        // min_color_dist_threshold nColorDistThreshold), BackgroundSubtractorLBSP.hpp:23-28
        out->desc_dist_threshold_offset = 4;
        out->min_color_dist_threshold = 30;
        out->bg_samples = 35;
        out->required_bg_samples = 2;
        out->samples_for_moving_avgs = 100;
        out->rel_lbsp_threshold = 0.333f;
        out->lbsp_threshold_offset = 0;
        out->default_median_blur_kernel_size = 9;
        out->seed = 0;
        out->device_id = 0;
        return LVBGS_OK;
    }
    if (algo == LVBGS_ALGO_VIBE) {
        // BackgroundSubtractorViBe.hpp:39-46 (min_color_dist_threshold carries nColorDistThreshold)
        out->desc_dist_threshold_offset = 0;
        out->min_color_dist_threshold = 20;
        out->bg_samples = 20;
        out->required_bg_samples = 2;
        out->samples_for_moving_avgs = 100;
        out->rel_lbsp_threshold = 0.333f;
        out->lbsp_threshold_offset = 0;
        out->default_median_blur_kernel_size = 9;
        out->seed = 0;
        out->device_id = 0;
        return LVBGS_OK;
    }
    if (algo != LVBGS_ALGO_SUBSENSE) return fail(nullptr, LVBGS_BAD_ARG, "unknown algorithm");
    out->desc_dist_threshold_offset = 3;
    out->min_color_dist_threshold = 30;
    out->bg_samples = 50;
    out->required_bg_samples = 2;
    out->samples_for_moving_avgs = 100;
    out->rel_lbsp_threshold = 0.333f;
    out->lbsp_threshold_offset = 0;
    out->default_median_blur_kernel_size = 9;
    out->seed = 0;
    out->device_id = 0;
    return LVBGS_OK;
}

lvbgs_status lvbgs_create(lvbgs_algo algo, const lvbgs_params* p, lvbgs_handle* out) {
    if (!out) return fail(nullptr, LVBGS_BAD_ARG, "null output handle");
    *out = nullptr;
    if (algo != LVBGS_ALGO_SUBSENSE && algo != LVBGS_ALGO_PAWCS && algo != LVBGS_ALGO_LOBSTER && algo != LVBGS_ALGO_VIBE &&
        algo != LVBGS_ALGO_PBAS)
        return fail(nullptr, LVBGS_BAD_ARG, "unknown algorithm");
    lvbgs_params prm;
    if (p) prm = *p;
    else lvbgs_default_params(algo, &prm);
    if (algo == LVBGS_ALGO_PAWCS) {
        // BackgroundSubtractorPAWCS.cpp:105 (max local and global word counts positive)
        if (prm.bg_samples / 2 == 0) return fail(nullptr, LVBGS_BAD_ARG, "max local/global word counts must be positive");
        if (prm.bg_samples / 2 > (size_t)kPwMaxLocal)
            return fail(nullptr, LVBGS_UNSUPPORTED, "this implementation supports at most 51 PAWCS words (25 local, 12 global)");
        prm.required_bg_samples = 0;
    }
    // BackgroundSubtractorSuBSENSE.cpp:76-77, BackgroundSubtractorLBSP.hpp:53
    if (prm.bg_samples == 0 || prm.required_bg_samples > prm.bg_samples)
        return fail(nullptr, LVBGS_BAD_ARG, "algo cannot require more sample matches than sample count in model");
    // ViBe's constructor checks the sample counts only (BackgroundSubtractorViBe.cpp:28); PBAS's also the
    // update rate (BackgroundSubtractorPBAS.cpp:31-32)
    if (algo == LVBGS_ALGO_PBAS && !(prm.update_rate > 0 && prm.update_rate <= 255))
        return fail(nullptr, LVBGS_BAD_ARG, "update rate must be in (0, 255]");
    if (algo != LVBGS_ALGO_VIBE && algo != LVBGS_ALGO_PBAS && prm.min_color_dist_threshold == 0 &&
        prm.desc_dist_threshold_offset == 0)
        return fail(nullptr, LVBGS_BAD_ARG, "distance thresholds must be positive values");
    if (!(prm.rel_lbsp_threshold >= 0)) return fail(nullptr, LVBGS_BAD_ARG, "relative threshold for LBSP features must be non-negative");
    if (prm.bg_samples > (size_t)kMaxSamples)
        return fail(nullptr, LVBGS_UNSUPPORTED, "this implementation supports at most 64 model samples");
    if (prm.samples_for_moving_avgs < 4 || prm.min_color_dist_threshold > 100000 || prm.desc_dist_threshold_offset > 100000)
        return fail(nullptr, LVBGS_UNSUPPORTED, "parameter outside the supported range");
    if (prm.default_median_blur_kernel_size < 1 || prm.default_median_blur_kernel_size > 31 ||
        (prm.default_median_blur_kernel_size % 2) == 0)
        return fail(nullptr, LVBGS_BAD_ARG, "median blur kernel size must be odd, between 1 and 31");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= prm.device_id || prm.device_id < 0) {
        cudaGetLastError();
        return fail(nullptr, LVBGS_DEVICE_ERROR, "no CUDA device with the requested id");
    }
    if (cudaSetDevice(prm.device_id) != cudaSuccess) return fail(nullptr, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    cudaFuncAttributes fa;
    if (cudaFuncGetAttributes(&fa, (const void*)lvbgs_k_eval) != cudaSuccess) {
        cudaGetLastError();
        return fail(nullptr, LVBGS_DEVICE_ERROR, "the library's sm_103a kernels cannot run on this device");
    }
    int coop = 0;
    cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, prm.device_id);
    if (!coop) return fail(nullptr, LVBGS_DEVICE_ERROR, "device does not support cooperative launches");
    {
        // exact division tables, once per device
        static std::mutex mu;
        static std::vector<int> done;
        std::lock_guard<std::mutex> lk(mu);
        if (std::find(done.begin(), done.end(), prm.device_id) == done.end()) {
            lvbgs_init_tables<<<1, 256>>>();
            if (cudaDeviceSynchronize() != cudaSuccess) {
                cudaGetLastError();
                return fail(nullptr, LVBGS_DEVICE_ERROR, "table initialization failed");
            }
            done.push_back(prm.device_id);
        }
    }
    lvbgs_ctx* h = new lvbgs_ctx();
    h->algo = algo;
    if (algo == LVBGS_ALGO_LOBSTER || algo == LVBGS_ALGO_VIBE || algo == LVBGS_ALGO_PBAS) h->lob = new LobState();
    h->prm = prm;
    h->device = prm.device_id;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete h;
        return fail(nullptr, LVBGS_DEVICE_ERROR, "stream creation failed");
    }
    *out = h;
    return LVBGS_OK;
}

lvbgs_status lvbgs_destroy(lvbgs_handle h) {
    if (!h) return LVBGS_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->dmem);
    h->ws.release();
    h->batchWs.release();
    if (h->h_flags) cudaFreeHost(h->h_flags);
    for (int g = 0; g < 3; ++g) {
        if (h->aux[g]) {
            cudaStreamSynchronize(h->aux[g]);
            cudaStreamDestroy(h->aux[g]);
        }
        if (h->evJoin[g]) cudaEventDestroy(h->evJoin[g]);
    }
    if (h->evFork) cudaEventDestroy(h->evFork);
    if (h->evPw) cudaEventDestroy(h->evPw);
    if (h->stream) cudaStreamDestroy(h->stream);
    if (h->lob) {
        lob_release(*h->lob);
        delete h->lob;
    }
    delete h;
    return LVBGS_OK;
}

lvbgs_status lvbgs_initialize(lvbgs_handle h, const uint8_t* img, int W, int H, int C, size_t stride, const uint8_t* roi) {
    if (!h) return fail(nullptr, LVBGS_BAD_ARG, "null handle");
    if (!img || W <= 0 || H <= 0) return fail(h, LVBGS_BAD_ARG, "provided image for initialization must be non-empty");
    if (C == 4) return fail(h, LVBGS_UNSUPPORTED, "8UC4 frames are not handled by SuBSENSE's apply() (1 or 3 channels)");
    if (C != 1 && C != 3) return fail(h, LVBGS_BAD_TYPE, "image must be of type 8UC1 or 8UC3");
    if ((size_t)W * H >= (1ull << 31)) return fail(h, LVBGS_UNSUPPORTED, "frame too large");
    if (cudaSetDevice(h->device) != cudaSuccess) return fail(h, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    const size_t npx = (size_t)W * H;
    const size_t row = (size_t)W * C;
    if (stride == 0) stride = row;
    if (stride < row) return fail(h, LVBGS_BAD_ARG, "image stride is smaller than width*channels");
    if (h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        // ViBe's and PBAS's initialize(img) take no ROI and use every pixel (BackgroundSubtractorViBe.cpp:57-75,
        // BackgroundSubtractorPBAS.cpp:61-109)
        if (roi) return fail(h, LVBGS_UNSUPPORTED, "ViBe and PBAS have no region of interest");
        return lob_initialize(h, img, W, H, C, stride, std::vector<uint8_t>(npx, 255), npx, npx);
    }
    // ROI handling (BackgroundSubtractionUtils.cpp:83-101, validateROI :28-36)
    std::vector<uint8_t> newroi(npx, 255);
    if (!roi && h->roi.size() == npx && h->roiW == W && h->roiH == H) {
        // no new ROI and the same size: the last validated ROI is reused (:86-87)
        newroi = h->roi;
    } else if (roi) {
        const bool devRoi = is_device_ptr(roi);
        std::vector<uint8_t> r(npx);
        if (devRoi) LV_CUDA(h, cudaMemcpy(r.data(), roi, npx, cudaMemcpyDeviceToHost), "roi download");
        else std::memcpy(r.data(), roi, npx);
        for (size_t i = 0; i < npx; ++i)
            if (r[i] != 0 && r[i] != 255) return fail(h, LVBGS_BAD_ARG, "provided ROI mat values must be 0 or 255 only");
        std::vector<uint8_t> d;
        host_dilate(r, d, W, H, kBorder);
        // `Mat / 2` is OpenCV's scaling expression, rounded half to even: 255 -> 128
        for (size_t i = 0; i < npx; ++i) newroi[i] = (uint8_t)(r[i] | ((d[i] + 1) / 2));
    }
    size_t orig = 0;
    for (size_t i = 0; i < npx; ++i) orig += newroi[i] != 0;
    if (orig == 0) return fail(h, LVBGS_BAD_ARG, "provided ROI mat contains no useful pixels");
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x)
            if (x < kBorder || y < kBorder || x >= W - kBorder || y >= H - kBorder) newroi[(size_t)y * W + x] = 0;
    size_t fin = 0;
    for (size_t i = 0; i < npx; ++i) fin += newroi[i] != 0;
    if (fin == 0)
        return fail(h, LVBGS_BAD_ARG, "provided ROI mat contains no useful pixels away from borders (descriptors will hit image bounds)");
    if (h->algo == LVBGS_ALGO_PAWCS) return pw_initialize(h, img, W, H, C, stride, newroi, orig, fin);
    if (h->algo == LVBGS_ALGO_LOBSTER) return lob_initialize(h, img, W, H, C, stride, newroi, orig, fin);
    // resolution-dependent parameters (BackgroundSubtractorSuBSENSE.cpp:112-128)
    StreamCtl ctl;
    std::memset(&ctl, 0, sizeof(ctl));
    const int area = W * H;
    if (orig >= npx / 2 && (int)npx >= 320 * 240) {
        ctl.lr_scaling = 1;
        ctl.auto_reset = 1;
        ctl.use3x3 = !(area > 320 * 240 * 2);
        int raw = (int)std::floor((float)area / (320 * 240) + 0.5f) + h->prm.default_median_blur_kernel_size;
        raw = std::min(raw, 14);
        ctl.median_k = (raw % 2) ? raw : raw - 1;
        ctl.t_lo = 2.0f;
        ctl.t_hi = 256.0f;
    } else {
        ctl.lr_scaling = 0;
        ctl.auto_reset = 0;
        ctl.use3x3 = 1;
        ctl.median_k = h->prm.default_median_blur_kernel_size;
        ctl.t_lo = 4.0f;
        ctl.t_hi = 512.0f;
    }
    const float rel = h->prm.rel_lbsp_threshold;
    for (int t = 0; t <= 255; ++t)
        ctl.lut[t] = C == 1 ? sat_round_u8(((float)t * rel + (float)h->prm.lbsp_threshold_offset) / 3)
                            : sat_round_u8((float)t * rel + (float)h->prm.lbsp_threshold_offset);
    ctl.n_rel = fin;
    ctl.orig_roi = orig;
    ctl.stamp_base = 1;
    frame_factors(1ull, (int)h->prm.samples_for_moving_avgs, &ctl.fLT, &ctl.fST, &ctl.bLT, &ctl.bST);
    // (re)allocate the device model
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaFree(h->dmem);
    h->dmem = nullptr;
    h->initialized = false;
    h->spilled = false;
    const Layout L = make_layout(W, H, C, h->prm.bg_samples);
    LV_CUDA(h, cudaMalloc(&h->dmem, L.total), "model allocation");
    h->persistBytes = L.persist;
    h->totalBytes = L.total;
    h->W = W;
    h->H = H;
    h->C = C;
    h->npx = npx;
    h->roi = newroi;
    h->roiW = W;
    h->roiH = H;
    h->n_rel = fin;
    h->orig_roi = orig;
    fill_pointers(h, L);
    fill_geometry(h);
    h->sd.lrScaling = ctl.lr_scaling;
    cudaStream_t st = h->stream;
    LV_CUDA(h, cudaMemsetAsync(h->dmem, 0, L.total, st), "model reset");
    LV_CUDA(h, cudaMemcpyAsync(h->sd.ctl, &ctl, sizeof(ctl), cudaMemcpyHostToDevice, st), "control upload");
    LV_CUDA(h, cudaMemcpyAsync(h->sd.roi, h->roi.data(), npx, cudaMemcpyHostToDevice, st), "roi upload");
    const uint8_t* dimg = nullptr;
    lvbgs_status s = stage_frame(h, img, stride, st, &dimg);
    if (s != LVBGS_OK) return s;
    lvbgs_init_maps<<<1024, 256, 0, st>>>(h->sd, dimg, ctl.t_lo);
    LV_CUDA(h, cudaGetLastError(), "init kernel launch");
    // refreshModel(1.0f) at frame 0 (BackgroundSubtractorSuBSENSE.cpp:184)
    lvbgs_refresh<<<1024, 256, 0, st>>>(h->sd, 0u, 0, (int)h->prm.bg_samples, 0, 0);
    LV_CUDA(h, cudaGetLastError(), "refresh kernel launch");
    LV_CUDA(h, h->ws.ensure(npx, 1), "workspace allocation");
    LV_CUDA(h, cudaStreamSynchronize(st), "initialization");
    h->initialized = true;
    return LVBGS_OK;
}

lvbgs_status lvbgs_apply(lvbgs_handle h, const uint8_t* img, size_t stride, uint8_t* mask, double lr, void* cuda_stream) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (!img) return fail(h, LVBGS_BAD_ARG, "null input image");
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : h->stream;
    if (h->algo == LVBGS_ALGO_PAWCS) return pw_apply(h, img, stride, mask, lr, st);
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        // BackgroundSubtractorLOBSTER.cpp:463, BackgroundSubtractorViBe.cpp:79: the rate is reinterpreted as an
        // integer and must be positive; PBAS's learningRateOverride replaces T(x) when positive (:174 / :402)
        if (h->algo != LVBGS_ALGO_PBAS && !(lr > 0))
            return fail(h, LVBGS_BAD_ARG, "learning rate must be a positive value; faster learning is achieved with smaller values");
        const uint8_t* dimg = nullptr;
        if ((s = stage_frame(h, img, stride, st, &dimg)) != LVBGS_OK) return s;
        const bool devMask = mask && is_device_ptr(mask);
        std::string err;
        s = lob_apply(*h->lob, dimg, devMask ? mask : h->d_mask, (mask && !devMask) ? mask : nullptr, lr, st, err);
        return s == LVBGS_OK ? s : fail(h, s, err);
    }
    const uint8_t* dimg = nullptr;
    if ((s = stage_frame(h, img, stride, st, &dimg)) != LVBGS_OK) return s;
    const bool devMask = mask_writable_by_device(mask);
    h->ws.h_streams.assign(1, h->sd);
    StreamDev& S = h->ws.h_streams[0];
    S.frame = dimg;
    S.maskOut = devMask ? mask : h->d_mask;
    set_lr(S, lr);
    if ((s = launch_tick(h, h->ws, 1, st)) != LVBGS_OK) return s;
    if (mask && !devMask) LV_CUDA(h, cudaMemcpyAsync(mask, h->d_mask, h->npx, cudaMemcpyDeviceToHost, st), "mask download");
    LV_CUDA(h, cudaStreamSynchronize(st), "frame step");
    return read_work_status(h, h->ws);
}

namespace {
// checks a batch (initialized handles on one device, each at most once)
lvbgs_status check_batch(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, bool allowPawcs) {
    if (!hs || !frames || n <= 0) return fail(nullptr, LVBGS_BAD_ARG, "empty batch");
    lvbgs_handle lead = hs[0];
    for (int i = 0; i < n; ++i) {
        lvbgs_status s = check_ready(hs[i]);
        if (s != LVBGS_OK) return s;
        if (hs[i]->device != lead->device) return fail(lead, LVBGS_BAD_ARG, "batched handles must share one device");
        if (!frames[i].image) return fail(hs[i], LVBGS_BAD_ARG, "null input image");
        if (hs[i]->algo != LVBGS_ALGO_SUBSENSE && !(allowPawcs && hs[i]->algo == LVBGS_ALGO_PAWCS))
            return fail(hs[i], LVBGS_UNSUPPORTED,
                        allowPawcs ? "batched frame steps are implemented for SuBSENSE and PAWCS streams"
                                   : "batch contexts run SuBSENSE streams");
        for (int j = 0; j < i; ++j)
            if (hs[j] == hs[i]) return fail(lead, LVBGS_BAD_ARG, "a handle appears twice in the batch");
    }
    return LVBGS_OK;
}
// stages the frames and fills the n stream descriptors of one batched tick
lvbgs_status prepare_batch(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, cudaStream_t st, StreamDev* out) {
    for (int i = 0; i < n; ++i) {
        lvbgs_handle h = hs[i];
        const uint8_t* dimg = nullptr;
        lvbgs_status s = stage_frame(h, frames[i].image, frames[i].stride, st, &dimg);
        if (s != LVBGS_OK) return s;
        out[i] = h->sd;
        StreamDev& S = out[i];
        S.frame = dimg;
        const bool devMask = mask_writable_by_device(frames[i].fgmask);
        S.maskOut = devMask ? frames[i].fgmask : h->d_mask;
        set_lr(S, frames[i].learning_rate);
    }
    return LVBGS_OK;
}
// enqueues the copies of the masks that go to host memory
lvbgs_status download_masks(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, cudaStream_t st) {
    for (int i = 0; i < n; ++i)
        if (frames[i].fgmask && !mask_writable_by_device(frames[i].fgmask))
            LV_CUDA(hs[0], cudaMemcpyAsync(frames[i].fgmask, hs[i]->d_mask, hs[i]->npx, cudaMemcpyDeviceToHost, st),
                    "mask download");
    return LVBGS_OK;
}
}  // namespace

namespace {
std::atomic<int> g_batch_groups{4};
constexpr int kMaxBatchGroups = 4;
constexpr int kSplitMinStreams = 8;
constexpr size_t kSplitMinPx = (size_t)4 << 20;

// Large batches run as G groups of about equal pixels (the largest streams first, each to the lightest
// group; the order within a group is the batch's): one group's latency-bound phases (the repair rounds,
// the hole-fill row walks) then overlap the other groups' work. Returns the number of groups (1: no
// split).
int split_batch(const lvbgs_handle* hs, int n, std::vector<std::vector<int>>& groups) {
    const int G = std::min(g_batch_groups.load(), n / (kSplitMinStreams / 2));
    size_t total = 0;
    for (int i = 0; i < n; ++i) total += hs[i]->npx;
    if (G < 2 || n < kSplitMinStreams || total < kSplitMinPx) return 1;
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return hs[a]->npx > hs[b]->npx; });
    std::vector<int> gof(n, 0);
    std::vector<size_t> load(G, 0);
    for (int i : order) {
        int g = 0;
        for (int k = 1; k < G; ++k)
            if (load[k] < load[g]) g = k;
        gof[i] = g;
        load[g] += hs[i]->npx;
    }
    groups.assign(G, std::vector<int>());
    for (int i = 0; i < n; ++i) groups[gof[i]].push_back(i);
    return G;
}

lvbgs_status batch_group(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, cudaStream_t st, int repairDiv) {
    lvbgs_handle lead = hs[0];
    Workspace& ws = lead->batchWs;
    ws.repairDiv = repairDiv;
    ws.h_streams.resize(n);
    lvbgs_status s = prepare_batch(hs, frames, n, st, ws.h_streams.data());
    if (s != LVBGS_OK) return s;
    if ((s = launch_tick(lead, ws, n, st)) != LVBGS_OK) return s;
    return download_masks(hs, frames, n, st);
}
}  // namespace

lvbgs_status lvbgs_set_batch_groups(int groups) {
    if (groups < 1 || groups > kMaxBatchGroups) return fail(nullptr, LVBGS_BAD_ARG, "batch groups must be 1..4");
    g_batch_groups = groups;
    return LVBGS_OK;
}

namespace {
// the SuBSENSE part of a batch: one sequence of phase kernels over its streams (split into concurrent
// groups when large)
lvbgs_status batch_apply_subsense(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, void* cuda_stream) {
    lvbgs_status s = LVBGS_OK;
    lvbgs_handle lead = hs[0];
    cudaSetDevice(lead->device);
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : lead->stream;
    std::vector<std::vector<int>> groups;
    const int G = split_batch(hs, n, groups);
    if (G == 1) return batch_group(hs, frames, n, st, 1);
    // group 0 runs on st, the others on the lead's further streams, forked from and joined back into
    // st; each group's cooperative repair grid takes 1/G of the co-resident blocks so that all fit
    if (!lead->evFork) LV_CUDA(lead, cudaEventCreateWithFlags(&lead->evFork, cudaEventDisableTiming), "event creation");
    for (int g = 0; g < G - 1; ++g) {
        if (!lead->aux[g]) LV_CUDA(lead, cudaStreamCreateWithFlags(&lead->aux[g], cudaStreamNonBlocking), "stream creation");
        if (!lead->evJoin[g])
            LV_CUDA(lead, cudaEventCreateWithFlags(&lead->evJoin[g], cudaEventDisableTiming), "event creation");
    }
    LV_CUDA(lead, cudaEventRecord(lead->evFork, st), "fork");
    for (int g = 0; g < G - 1; ++g) LV_CUDA(lead, cudaStreamWaitEvent(lead->aux[g], lead->evFork, 0), "fork");
    std::vector<lvbgs_handle> hg;
    std::vector<lvbgs_frame> fg;
    for (int g = 0; g < G; ++g) {
        hg.clear();
        fg.clear();
        for (int i : groups[g]) {
            hg.push_back(hs[i]);
            fg.push_back(frames[i]);
        }
        if ((s = batch_group(hg.data(), fg.data(), (int)hg.size(), g == 0 ? st : lead->aux[g - 1], G)) != LVBGS_OK)
            return s;
    }
    for (int g = 0; g < G - 1; ++g) {
        LV_CUDA(lead, cudaEventRecord(lead->evJoin[g], lead->aux[g]), "join");
        LV_CUDA(lead, cudaStreamWaitEvent(st, lead->evJoin[g], 0), "join");
    }
    return LVBGS_OK;
}

}  // namespace

// A batch may mix SuBSENSE and PAWCS streams. The SuBSENSE streams run as one batched frame step on the
// caller's stream; each PAWCS stream's frame step runs on the handle's own stream (forked from the
// caller's and joined back into it), all of them in flight together: the host waits for their
// fixed-point rounds in turn, so the call returns once every PAWCS step is enqueued to its end.
lvbgs_status lvbgs_batch_apply(const lvbgs_handle* hs, const lvbgs_frame* frames, int n, void* cuda_stream) {
    lvbgs_status s = check_batch(hs, frames, n, true);
    if (s != LVBGS_OK) return s;
    std::vector<lvbgs_handle> sub, pw;
    std::vector<lvbgs_frame> fsub, fpw;
    for (int i = 0; i < n; ++i) {
        if (hs[i]->algo == LVBGS_ALGO_PAWCS) {
            pw.push_back(hs[i]);
            fpw.push_back(frames[i]);
        } else {
            sub.push_back(hs[i]);
            fsub.push_back(frames[i]);
        }
    }
    if (pw.empty()) return batch_apply_subsense(hs, frames, n, cuda_stream);
    lvbgs_handle lead = hs[0];
    cudaSetDevice(lead->device);
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : lead->stream;
    for (lvbgs_handle h : pw)
        if (!h->evPw) LV_CUDA(h, cudaEventCreateWithFlags(&h->evPw, cudaEventDisableTiming), "event creation");
    // fork: every PAWCS step starts after the work the caller enqueued on st
    LV_CUDA(lead, cudaEventRecord(pw[0]->evPw, st), "fork");
    for (lvbgs_handle h : pw) LV_CUDA(h, cudaStreamWaitEvent(h->stream, pw[0]->evPw, 0), "fork");
    std::vector<char> live(pw.size(), 0);
    lvbgs_status first = LVBGS_OK;
    for (size_t i = 0; i < pw.size(); ++i) {
        s = pw_begin(pw[i], fpw[i].image, fpw[i].stride, fpw[i].fgmask, fpw[i].learning_rate, pw[i]->stream);
        if (s == LVBGS_OK) live[i] = 1;
        else {
            pw[i]->pws.active = false;
            if (first == LVBGS_OK) first = s;
        }
    }
    if (!sub.empty() && first == LVBGS_OK) first = batch_apply_subsense(sub.data(), fsub.data(), (int)sub.size(), st);
    // the PAWCS steps advance in turn until each is over (every step in flight is run to its end, also
    // after an error, so that no handle is left with a step in flight)
    for (bool any = true; any;) {
        any = false;
        for (size_t i = 0; i < pw.size(); ++i) {
            if (!live[i]) continue;
            bool done = false;
            s = pw_advance(pw[i], done);
            if (done) {
                live[i] = 0;
                if (s != LVBGS_OK && first == LVBGS_OK) first = s;
            } else {
                any = true;
            }
        }
    }
    // join: the caller's stream waits for every PAWCS step (they are over; this orders later work)
    for (lvbgs_handle h : pw) {
        LV_CUDA(h, cudaEventRecord(h->evPw, h->stream), "join");
        LV_CUDA(lead, cudaStreamWaitEvent(st, h->evPw, 0), "join");
    }
    return first;
}

lvbgs_status lvbgs_batch_wait(const lvbgs_handle* handles, int n_all, void* cuda_stream) {
    if (!handles || n_all <= 0) return fail(nullptr, LVBGS_BAD_ARG, "empty batch");
    lvbgs_handle lead0 = handles[0];
    cudaSetDevice(lead0->device);
    cudaStream_t st = cuda_stream ? (cudaStream_t)cuda_stream : lead0->stream;
    LV_CUDA(lead0, cudaStreamSynchronize(st), "batched frame step");
    // the device status of the SuBSENSE part (the PAWCS steps reported theirs in lvbgs_batch_apply)
    std::vector<lvbgs_handle> sub;
    for (int i = 0; i < n_all; ++i)
        if (handles[i] && handles[i]->algo != LVBGS_ALGO_PAWCS) sub.push_back(handles[i]);
    if (sub.empty()) return LVBGS_OK;
    const lvbgs_handle* hs = sub.data();
    const int n = (int)sub.size();
    lvbgs_handle lead = hs[0];
    std::vector<std::vector<int>> groups;
    const int G = split_batch(hs, n, groups);
    if (G == 1) return read_work_status(lead, lead->batchWs);
    for (int g = 0; g < G; ++g) {
        // the status of each group's work area (the groups' leads)
        const lvbgs_handle gl = hs[groups[g][0]];
        lvbgs_status s = read_work_status(gl, gl->batchWs);
        if (s != LVBGS_OK) return s;
    }
    return LVBGS_OK;
}

// ---- batch contexts: a work area owned apart from the streams, with ticks kept in flight ----
struct lvbgs_batch_ctx {
    int device = 0;
    Workspace ws;
    cudaStream_t stream = nullptr;  // the stream of the ticks in flight
    struct Slot {
        StreamDev* hS = nullptr;             // pinned descriptor table of the tick
        unsigned long long* hDs = nullptr;   // pinned down-sampling offsets
        TickWork* hWork = nullptr;           // pinned copy of the tick's status
        int cap = 0;
        cudaEvent_t done = nullptr;
        uint64_t ticket = 0;
        bool busy = false;
    } slots[LVBGS_BATCH_MAX_INFLIGHT];
    uint64_t next = 1;
    int inflight = 0;
};

namespace {
void free_slot(lvbgs_batch_ctx::Slot& sl) {
    cudaFreeHost(sl.hS);
    cudaFreeHost(sl.hDs);
    sl.hS = nullptr;
    sl.hDs = nullptr;
    sl.cap = 0;
}
cudaError_t grow_slot(lvbgs_batch_ctx::Slot& sl, int n) {
    if (n <= sl.cap) return cudaSuccess;
    free_slot(sl);
    const int cap = std::max(n + n / 2, 16);
    cudaError_t e = cudaHostAlloc((void**)&sl.hS, sizeof(StreamDev) * cap, cudaHostAllocDefault);
    if (e == cudaSuccess) e = cudaHostAlloc((void**)&sl.hDs, sizeof(unsigned long long) * (cap + 1), cudaHostAllocDefault);
    if (e == cudaSuccess) sl.cap = cap;
    return e;
}
}  // namespace

lvbgs_status lvbgs_batch_create(int device_id, size_t reserve_px, int reserve_streams, lvbgs_batch* out) {
    if (!out) return fail(nullptr, LVBGS_BAD_ARG, "null output");
    *out = nullptr;
    if (reserve_streams < 0) return fail(nullptr, LVBGS_BAD_ARG, "negative stream reservation");
    if (cudaSetDevice(device_id) != cudaSuccess) return fail(nullptr, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    lvbgs_batch b = new lvbgs_batch_ctx();
    b->device = device_id;
    cudaError_t e = b->ws.ensure(std::max<size_t>(reserve_px, 1), std::max(reserve_streams, 1));
    for (auto& sl : b->slots) {
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaHostAlloc((void**)&sl.hWork, sizeof(TickWork), cudaHostAllocDefault);
        if (e == cudaSuccess) e = grow_slot(sl, std::max(reserve_streams, 1));
    }
    if (e != cudaSuccess) {
        lvbgs_batch_destroy(b);
        return cuda_fail(nullptr, e, "batch context allocation");
    }
    *out = b;
    return LVBGS_OK;
}

lvbgs_status lvbgs_batch_destroy(lvbgs_batch b) {
    if (!b) return LVBGS_OK;
    cudaSetDevice(b->device);
    for (auto& sl : b->slots)
        if (sl.busy && sl.done) cudaEventSynchronize(sl.done);
    for (auto& sl : b->slots) {
        free_slot(sl);
        cudaFreeHost(sl.hWork);
        if (sl.done) cudaEventDestroy(sl.done);
    }
    b->ws.release();
    delete b;
    return LVBGS_OK;
}

lvbgs_status lvbgs_batch_reserve(lvbgs_batch b, size_t px, int n_streams) {
    if (!b || n_streams < 0) return fail(nullptr, LVBGS_BAD_ARG, "bad argument");
    cudaSetDevice(b->device);
    if (b->inflight > 0 && (px > b->ws.cap || n_streams > b->ws.nStreamsCap))
        return fail(nullptr, LVBGS_BAD_ARG, "cannot grow a batch context with ticks in flight");
    LV_CUDA(nullptr, b->ws.ensure(std::max<size_t>(px, 1), std::max(n_streams, 1)), "batch workspace allocation");
    return LVBGS_OK;
}

lvbgs_status lvbgs_batch_set_repair_share(lvbgs_batch b, int divisor) {
    if (!b || divisor < 1 || divisor > 64) return fail(nullptr, LVBGS_BAD_ARG, "repair share divisor must be 1..64");
    b->ws.repairDiv = divisor;
    return LVBGS_OK;
}

lvbgs_status lvbgs_batch_submit(lvbgs_batch b, const lvbgs_handle* hs, const lvbgs_frame* frames, int n,
                                void* cuda_stream, uint64_t* ticket) {
    if (!b || !ticket) return fail(nullptr, LVBGS_BAD_ARG, "null argument");
    lvbgs_status s = check_batch(hs, frames, n, false);
    if (s != LVBGS_OK) return s;
    lvbgs_handle lead = hs[0];
    if (lead->device != b->device) return fail(lead, LVBGS_BAD_ARG, "batch context and handles are on different devices");
    cudaSetDevice(b->device);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    if (!st) return fail(lead, LVBGS_BAD_ARG, "batched ticks of a context need an explicit CUDA stream");
    if (b->inflight > 0 && st != b->stream)
        return fail(lead, LVBGS_BAD_ARG, "ticks in flight on one batch context must share one CUDA stream");
    lvbgs_batch_ctx::Slot& sl = b->slots[b->next % LVBGS_BATCH_MAX_INFLIGHT];
    if (sl.busy) return fail(lead, LVBGS_BAD_ARG, "too many ticks in flight: complete the oldest first");
    size_t px = 0;
    for (int i = 0; i < n; ++i) px += hs[i]->npx;
    if (b->inflight > 0 && (px > b->ws.cap || n > b->ws.nStreamsCap))
        return fail(lead, LVBGS_BAD_ARG, "batch exceeds the context's reservation while ticks are in flight");
    LV_CUDA(lead, grow_slot(sl, n), "descriptor table allocation");
    if ((s = prepare_batch(hs, frames, n, st, sl.hS)) != LVBGS_OK) return s;
    if ((s = launch_tick(lead, b->ws, n, st, sl.hS, sl.hDs)) != LVBGS_OK) return s;
    if ((s = download_masks(hs, frames, n, st)) != LVBGS_OK) return s;
    LV_CUDA(lead, cudaMemcpyAsync(sl.hWork, b->ws.work, sizeof(TickWork), cudaMemcpyDeviceToHost, st), "status copy");
    LV_CUDA(lead, cudaEventRecord(sl.done, st), "completion event");
    sl.ticket = b->next++;
    sl.busy = true;
    b->stream = st;
    ++b->inflight;
    *ticket = sl.ticket;
    return LVBGS_OK;
}

int lvbgs_batch_query(lvbgs_batch b, uint64_t ticket) {
    if (!b) return -1;
    lvbgs_batch_ctx::Slot& sl = b->slots[ticket % LVBGS_BATCH_MAX_INFLIGHT];
    if (!sl.busy || sl.ticket != ticket) return -1;
    cudaSetDevice(b->device);
    const cudaError_t e = cudaEventQuery(sl.done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return -1;
}

lvbgs_status lvbgs_batch_complete(lvbgs_batch b, uint64_t ticket) {
    if (!b) return fail(nullptr, LVBGS_BAD_ARG, "null batch context");
    lvbgs_batch_ctx::Slot& sl = b->slots[ticket % LVBGS_BATCH_MAX_INFLIGHT];
    if (!sl.busy || sl.ticket != ticket) return fail(nullptr, LVBGS_BAD_ARG, "unknown or already completed tick");
    cudaSetDevice(b->device);
    const cudaError_t e = cudaEventSynchronize(sl.done);
    sl.busy = false;
    --b->inflight;
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "batched frame step");
    return status_from_work(nullptr, *sl.hWork);
}

lvbgs_status lvbgs_get_background(lvbgs_handle h, uint8_t* out) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (!out) return fail(h, LVBGS_BAD_ARG, "null output");
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        std::string err;
        s = lob_background(*h->lob, out, false, h->stream, err);
        return s == LVBGS_OK ? s : fail(h, s, err);
    }
    if (h->algo == LVBGS_ALGO_PAWCS) {
        const bool dev = is_device_ptr(out);
        uint8_t* d = dev ? out : h->d_frame;
        if (h->C == 3) pw3_k_background<<<512, 256, 0, h->stream>>>(h->pd, (int)(h->pw_frames & 1ull), d, nullptr);
        else pw_k_background<<<512, 256, 0, h->stream>>>(h->pd, (int)(h->pw_frames & 1ull), d, nullptr);
        LV_CUDA(h, cudaGetLastError(), "background kernel");
        if (!dev) LV_CUDA(h, cudaMemcpyAsync(out, d, h->npx * h->C, cudaMemcpyDeviceToHost, h->stream), "download");
        LV_CUDA(h, cudaStreamSynchronize(h->stream), "background image");
        return LVBGS_OK;
    }
    const bool dev = is_device_ptr(out);
    uint8_t* d = dev ? out : h->d_frame;
    lvbgs_background<<<512, 256, 0, h->stream>>>(h->sd, d, nullptr);
    LV_CUDA(h, cudaGetLastError(), "background kernel");
    if (!dev) LV_CUDA(h, cudaMemcpyAsync(out, d, h->npx * h->C, cudaMemcpyDeviceToHost, h->stream), "download");
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "background image");
    return LVBGS_OK;
}

lvbgs_status lvbgs_get_background_descriptors(lvbgs_handle h, uint16_t* out) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (!out) return fail(h, LVBGS_BAD_ARG, "null output");
    if (h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS)
        return fail(h, LVBGS_UNSUPPORTED, "ViBe and PBAS keep no descriptors");
    if (h->algo == LVBGS_ALGO_LOBSTER) {
        std::string err;
        s = lob_background(*h->lob, out, true, h->stream, err);
        return s == LVBGS_OK ? s : fail(h, s, err);
    }
    uint16_t* d = nullptr;
    LV_CUDA(h, cudaMallocAsync((void**)&d, h->npx * h->C * 2, h->stream), "temporary allocation");
    if (h->algo == LVBGS_ALGO_PAWCS && h->C == 3)
        pw3_k_background<<<512, 256, 0, h->stream>>>(h->pd, (int)(h->pw_frames & 1ull), nullptr, d);
    else if (h->algo == LVBGS_ALGO_PAWCS)
        pw_k_background<<<512, 256, 0, h->stream>>>(h->pd, (int)(h->pw_frames & 1ull), nullptr, d);
    else lvbgs_background<<<512, 256, 0, h->stream>>>(h->sd, nullptr, d);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, h->npx * h->C * 2, cudaMemcpyDefault, h->stream);
    cudaFreeAsync(d, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return cuda_fail(h, e, "background descriptors");
    return LVBGS_OK;
}

lvbgs_status lvbgs_refresh_model(lvbgs_handle h, float frac, int force) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (h->algo == LVBGS_ALGO_PAWCS)
        return fail(h, LVBGS_BAD_ARG, "PAWCS's refreshModel takes (base occurrences, decrement fraction, force): use lvbgs_pawcs_refresh_model");
    if (h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS)
        return fail(h, LVBGS_UNSUPPORTED, "ViBe and PBAS have no refreshModel");
    if (!(frac > 0.0f && frac <= 1.0f)) return fail(h, LVBGS_BAD_ARG, "model refresh must be given as a non-null fraction");
    if (h->algo == LVBGS_ALGO_LOBSTER) {
        std::string err;
        s = lob_refresh(*h->lob, frac, force ? 1 : 0, h->stream, err);
        return s == LVBGS_OK ? s : fail(h, s, err);
    }
    StreamCtl ctl;
    LV_CUDA(h, cudaMemcpy(&ctl, h->sd.ctl, sizeof(ctl), cudaMemcpyDeviceToHost), "control read");
    const size_t N = h->prm.bg_samples;
    const size_t nref = frac < 1.0f ? (size_t)(frac * (float)N) : N;
    size_t start = 0;
    if (frac < 1.0f) {
        // frame-level draw (sentinel pixel) of nRefreshSampleStartPos (:86)
        const uint32_t k = ctl.ksent++;
        uint32_t c[4] = {k >> 2, kSentinelPx, (uint32_t)ctl.frame_idx, 0u};
        philox4x32_10(c, (uint32_t)h->prm.seed, (uint32_t)(h->prm.seed >> 32));
        start = (size_t)(c[k & 3u] & 0x7fffffffu) % N;
        LV_CUDA(h, cudaMemcpy(&h->sd.ctl->ksent, &ctl.ksent, sizeof(ctl.ksent), cudaMemcpyHostToDevice), "control write");
    }
    lvbgs_refresh<<<1024, 256, 0, h->stream>>>(h->sd, (uint32_t)ctl.frame_idx, (int)start, (int)nref, force ? 1 : 0,
                                               (int)(ctl.frame_idx & 1ull));
    LV_CUDA(h, cudaGetLastError(), "refresh kernel");
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "refresh");
    return LVBGS_OK;
}

lvbgs_status lvbgs_set_automatic_model_reset(lvbgs_handle h, int enabled) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    const int v = enabled ? 1 : 0;
    // LOBSTER keeps the flag of its base class but has no automatic model reset; ViBe and PBAS have neither
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) return LVBGS_OK;
    LV_CUDA(h, cudaMemcpy(&h->sd.ctl->auto_reset, &v, sizeof(v), cudaMemcpyHostToDevice), "control write");
    return LVBGS_OK;
}

// getDefaultLearningRate(): LOBSTER's BGSLOBSTER_DEFAULT_LEARNING_RATE (BackgroundSubtractorLOBSTER.hpp:31,57);
// 0 (the internal T(x)) for the others
double lvbgs_get_default_learning_rate(lvbgs_handle h) {
    if (!h) return 0.0;
    // BGSLOBSTER_DEFAULT_LEARNING_RATE and BGSVIBE_DEFAULT_LEARNING_RATE (BackgroundSubtractorViBe.hpp:46)
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE) return 16.0;
    // BGSPBAS_DEFAULT_LEARNING_RATE_OVERRIDE (BackgroundSubtractorPBAS.hpp:57): no override
    if (h->algo == LVBGS_ALGO_PBAS) return -1.0;
    return 0.0;
}

lvbgs_status lvbgs_set_roi(lvbgs_handle h, const uint8_t* roi, int width, int height) {
    if (!h || !roi || width <= 0 || height <= 0) return fail(h, LVBGS_BAD_ARG, "null or empty ROI");
    if (h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS)
        return fail(h, LVBGS_UNSUPPORTED, "ViBe and PBAS have no region of interest");
    const size_t npx = (size_t)width * height;
    std::vector<uint8_t> r(npx);
    if (is_device_ptr(roi)) LV_CUDA(h, cudaMemcpy(r.data(), roi, npx, cudaMemcpyDeviceToHost), "roi download");
    else std::memcpy(r.data(), roi, npx);
    // validateROI (:28-36): only [2, W-2) x [2, H-2) may stay in the ROI
    for (int y = 0; y < height; ++y)
        for (int x = 0; x < width; ++x)
            if (x < kBorder || y < kBorder || x >= width - kBorder || y >= height - kBorder) r[(size_t)y * width + x] = 0;
    size_t nz = 0;
    for (size_t i = 0; i < npx; ++i) nz += r[i] != 0;
    if (nz == 0) return fail(h, LVBGS_BAD_ARG, "provided ROI must have at least one valid pixel");
    if (h->initialized) {
        // re-initialize from the latest background image with the new ROI (:40-44)
        if (width != h->W || height != h->H)
            return fail(h, LVBGS_BAD_SIZE, "provided ROI mat size must be equal to the init frame size");
        std::vector<uint8_t> bg(npx * h->C);
        lvbgs_status s = lvbgs_get_background(h, bg.data());
        if (s != LVBGS_OK) return s;
        return lvbgs_initialize(h, bg.data(), width, height, h->C, 0, r.data());
    }
    h->roi = r;
    h->roiW = width;
    h->roiH = height;
    return LVBGS_OK;
}

lvbgs_status lvbgs_get_roi(lvbgs_handle h, uint8_t* out) {
    if (!h || !out) return fail(h, LVBGS_BAD_ARG, "null argument");
    if (!h->initialized) return fail(h, LVBGS_NOT_INITIALIZED, "algo must be initialized first");
    std::memcpy(out, h->roi.data(), h->npx);
    return LVBGS_OK;
}

lvbgs_status lvbgs_get_size(lvbgs_handle h, int* w, int* hh, int* c) {
    if (!h) return fail(nullptr, LVBGS_BAD_ARG, "null handle");
    if (!h->initialized) return fail(h, LVBGS_NOT_INITIALIZED, "algo must be initialized first");
    if (w) *w = h->W;
    if (hh) *hh = h->H;
    if (c) *c = h->C;
    return LVBGS_OK;
}

size_t lvbgs_state_bytes(lvbgs_algo algo, int W, int H, int C, size_t N) {
    if (algo == LVBGS_ALGO_PAWCS && W > 0 && H > 0 && (C == 1 || C == 3)) {
        lvbgs_params prm;
        lvbgs_default_params(LVBGS_ALGO_PAWCS, &prm);
        if (N) prm.bg_samples = N;
        const PwGeom g = pw_geometry(prm, (size_t)W * H, (size_t)W * H, C);
        return pw_layout(W, H, C, g.L, g.G).persist;
    }
    if (algo != LVBGS_ALGO_SUBSENSE || W <= 0 || H <= 0 || (C != 1 && C != 3)) return 0;
    return make_layout(W, H, C, N ? N : 50).persist;
}

size_t lvbgs_device_bytes(lvbgs_algo algo, int W, int H, int C, size_t N) {
    if (algo == LVBGS_ALGO_PAWCS && W > 0 && H > 0 && (C == 1 || C == 3)) {
        lvbgs_params prm;
        lvbgs_default_params(LVBGS_ALGO_PAWCS, &prm);
        if (N) prm.bg_samples = N;
        const PwGeom g = pw_geometry(prm, (size_t)W * H, (size_t)W * H, C);
        return pw_layout(W, H, C, g.L, g.G).total;
    }
    if (algo != LVBGS_ALGO_SUBSENSE || W <= 0 || H <= 0 || (C != 1 && C != 3)) return 0;
    // model and scratch block, plus the handle's own workspace (status, one descriptor table,
    // four repair lists of one entry per pixel)
    const size_t npx = (size_t)W * H;
    return make_layout(W, H, C, N ? N : 50).total + sizeof(TickWork) + 8 * sizeof(StreamDev) +
           9 * sizeof(unsigned long long) + 4 * sizeof(unsigned long long) * npx;
}

lvbgs_status lvbgs_spill(lvbgs_handle h, void* host, size_t bytes) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS)
        return fail(h, LVBGS_UNSUPPORTED, "spilling is implemented for SuBSENSE and PAWCS streams");
    if (!host || bytes < h->persistBytes) return fail(h, LVBGS_BAD_ARG, "spill buffer is smaller than lvbgs_state_bytes()");
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "spill");
    LV_CUDA(h, cudaMemcpy(host, h->dmem, h->persistBytes, cudaMemcpyDeviceToHost), "spill copy");
    cudaFree(h->dmem);
    h->dmem = nullptr;
    h->ws.release();
    h->batchWs.release();
    h->spilled = true;
    return LVBGS_OK;
}

lvbgs_status lvbgs_restore(lvbgs_handle h, const void* host, size_t bytes) {
    if (!h || !host) return fail(h, LVBGS_BAD_ARG, "null argument");
    if (!h->initialized || !h->spilled) return fail(h, LVBGS_NOT_INITIALIZED, "stream is not spilled");
    if (bytes < h->persistBytes) return fail(h, LVBGS_BAD_ARG, "restore buffer is smaller than lvbgs_state_bytes()");
    cudaSetDevice(h->device);
    if (h->algo == LVBGS_ALGO_PAWCS) {
        // PAWCS: the persistent prefix of the layout holds every cross-frame array (control blocks,
        // word planes, feedback and mask maps, sort tables, spatial word maps); the rest is per-frame
        // scratch, and the device descriptors are rebuilt from the handle's parameters
        const int L = h->pd.L, G = h->pd.G;
        const PwLayout Lo = pw_layout(h->W, h->H, h->C, L, G);
        LV_CUDA(h, cudaMalloc(&h->dmem, Lo.total), "model allocation");
        LV_CUDA(h, cudaMemcpy(h->dmem, host, h->persistBytes, cudaMemcpyHostToDevice), "restore copy");
        LV_CUDA(h, cudaMemset(h->dmem + h->persistBytes, 0, Lo.total - h->persistBytes), "scratch reset");
        pw_fill(h, Lo, L, G);
        lvbgs_status s = pw_upload_desc(h, h->stream);
        if (s != LVBGS_OK) return s;
        LV_CUDA(h, cudaStreamSynchronize(h->stream), "restore");
        h->spilled = false;
        return LVBGS_OK;
    }
    const Layout L = make_layout(h->W, h->H, h->C, h->prm.bg_samples);
    LV_CUDA(h, cudaMalloc(&h->dmem, L.total), "model allocation");
    LV_CUDA(h, cudaMemcpy(h->dmem, host, h->persistBytes, cudaMemcpyHostToDevice), "restore copy");
    LV_CUDA(h, cudaMemset(h->dmem + h->persistBytes, 0, L.total - h->persistBytes), "scratch reset");
    fill_pointers(h, L);
    // repair stamps restart from zero, so the stamp generation restarts above them
    const unsigned int one = 1;
    LV_CUDA(h, cudaMemcpy(&h->sd.ctl->stamp_base, &one, sizeof(one), cudaMemcpyHostToDevice), "control write");
    LV_CUDA(h, h->ws.ensure(h->npx, 1), "workspace allocation");
    h->spilled = false;
    return LVBGS_OK;
}

lvbgs_status lvbgs_lbsp_compute2(const uint8_t* img, int W, int H, int C, long absThr, float rel, size_t off,
                                 uint16_t* desc, int device_id) {
    if (!img || !desc || W <= 0 || H <= 0) return fail(nullptr, LVBGS_BAD_ARG, "input image must be non-empty");
    if (C != 1 && C != 3) return fail(nullptr, LVBGS_BAD_TYPE, "input image must be of type 8UC1/8UC3");
    if (absThr < 0 && !(rel >= 0)) return fail(nullptr, LVBGS_BAD_ARG, "relative LBSP threshold must be non-negative");
    if (cudaSetDevice(device_id) != cudaSuccess) return fail(nullptr, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    const size_t n = (size_t)W * H * C;
    uint8_t* di = nullptr;
    uint16_t* dd = nullptr;
    LV_CUDA(nullptr, cudaMalloc(&di, n), "allocation");
    cudaError_t e = cudaMalloc(&dd, n * 2);
    if (e == cudaSuccess) e = cudaMemcpy(di, img, n, cudaMemcpyDefault);
    if (e == cudaSuccess) e = cudaMemcpy(dd, desc, n * 2, cudaMemcpyDefault);  // border keeps the caller's content
    if (e == cudaSuccess) {
        const int thr = absThr < 0 ? -1 : (int)std::min<long>(absThr, 255);
        lvbgs_lbsp_dense<<<256, 256>>>(di, W, H, C, thr, rel, (unsigned)off, dd);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(desc, dd, n * 2, cudaMemcpyDefault);
    cudaFree(di);
    cudaFree(dd);
    if (e != cudaSuccess) return cuda_fail(nullptr, e, "LBSP extraction");
    return LVBGS_OK;
}

const char* lvbgs_last_error(lvbgs_handle h) {
    if (h) return h->err.c_str();
    std::lock_guard<std::mutex> lk(g_err_mu);
    static thread_local std::string copy;
    copy = g_err;
    return copy.c_str();
}

lvbgs_status lvbgs_debug_map_bytes(lvbgs_handle h, int which, size_t* bytes) {
    if (!h || !bytes) return fail(h, LVBGS_BAD_ARG, "null argument");
    if (!h->initialized) return fail(h, LVBGS_NOT_INITIALIZED, "algo must be initialized first");
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        *bytes = lob_map_bytes(*h->lob, which);
        return *bytes ? LVBGS_OK : fail(h, LVBGS_BAD_ARG, "map not kept by this algorithm");
    }
    const size_t npx = h->npx, C = (size_t)h->C, N = h->prm.bg_samples;
    const size_t nds = (size_t)h->sd.dsW * h->sd.dsH * C;
    if (which >= LVBGS_MAP_R && which <= LVBGS_MAP_FIN_ST) *bytes = npx * 4;
    else if (which >= LVBGS_MAP_UNSTABLE && which <= LVBGS_MAP_ROI) *bytes = npx;
    else if (which == LVBGS_MAP_LAST_COLOR) *bytes = npx * C;
    else if (which == LVBGS_MAP_LAST_DESC) *bytes = npx * C * 2;
    else if (which == LVBGS_MAP_SAMPLE_COLOR) *bytes = N * npx * C;
    else if (which == LVBGS_MAP_SAMPLE_DESC) *bytes = N * npx * C * 2;
    else if (which == LVBGS_MAP_DS_LT || which == LVBGS_MAP_DS_ST) *bytes = nds * 4;
    else if (which == LVBGS_MAP_LUT) *bytes = 256;
    else return fail(h, LVBGS_BAD_ARG, "unknown map id");
    return LVBGS_OK;
}

lvbgs_status lvbgs_debug_get_map(lvbgs_handle h, int which, void* out, size_t bytes) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    size_t need = 0;
    if ((s = lvbgs_debug_map_bytes(h, which, &need)) != LVBGS_OK) return s;
    if (!out || bytes < need) return fail(h, LVBGS_BAD_ARG, "output buffer too small");
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        std::string err;
        s = lob_get_map(*h->lob, which, out, bytes, h->stream, err);
        return s == LVBGS_OK ? s : fail(h, s, err);
    }
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "sync");
    StreamCtl ctl;
    LV_CUDA(h, cudaMemcpy(&ctl, h->sd.ctl, sizeof(ctl), cudaMemcpyDeviceToHost), "control read");
    const int cur = (int)(ctl.frame_idx & 1ull);
    const size_t npx = h->npx, C = (size_t)h->C, N = h->prm.bg_samples;
    const StreamDev& S = h->sd;
    const void* src = nullptr;
    if (which >= LVBGS_MAP_R && which <= LVBGS_MAP_FIN_ST)
        src = S.fm + (size_t)cur * kNumFloatMaps * npx + (size_t)(which - LVBGS_MAP_R) * npx;
    else if (which == LVBGS_MAP_UNSTABLE) src = S.unst + (size_t)cur * npx;
    else if (which == LVBGS_MAP_BLINKS) src = S.blinks;
    else if (which == LVBGS_MAP_LAST_RAW_FG) src = S.lastRawFG;
    else if (which == LVBGS_MAP_LAST_FG) src = S.lastFG;
    else if (which == LVBGS_MAP_LAST_FG_DIL_INV) src = S.dilInv;
    else if (which == LVBGS_MAP_LAST_RAW_BLINK) src = S.lastRawBlink;
    else if (which == LVBGS_MAP_ROI) src = S.roi;
    else if (which == LVBGS_MAP_LAST_COLOR) src = S.lastCol + (size_t)cur * npx * C;
    else if (which == LVBGS_MAP_LAST_DESC) src = S.lastDesc + (size_t)cur * npx * C;
    else if (which == LVBGS_MAP_DS_LT) src = S.dsLT;
    else if (which == LVBGS_MAP_DS_ST) src = S.dsST;
    else if (which == LVBGS_MAP_LUT) {
        std::memcpy(out, ctl.lut, 256);
        return LVBGS_OK;
    }
    if (src) {
        LV_CUDA(h, cudaMemcpy(out, src, need, cudaMemcpyDeviceToHost), "map download");
        return LVBGS_OK;
    }
    // sample images: unpack the planes into the reference's N images
    uint8_t* dcol = nullptr;
    uint16_t* ddesc = nullptr;
    LV_CUDA(h, cudaMalloc(&dcol, N * npx * C), "temporary allocation");
    cudaError_t e = cudaMalloc(&ddesc, N * npx * C * 2);
    if (e == cudaSuccess) {
        lvbgs_unpack_samples<<<1024, 256>>>(h->sd, dcol, ddesc);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        if (which == LVBGS_MAP_SAMPLE_COLOR) e = cudaMemcpy(out, dcol, need, cudaMemcpyDeviceToHost);
        else e = cudaMemcpy(out, ddesc, need, cudaMemcpyDeviceToHost);
    }
    cudaFree(dcol);
    cudaFree(ddesc);
    if (e != cudaSuccess) return cuda_fail(h, e, "sample download");
    return LVBGS_OK;
}

lvbgs_status lvbgs_debug_set_timing(lvbgs_handle h, int batched, int n_ticks) {
    if (!h || n_ticks < 0) return fail(h, LVBGS_BAD_ARG, "bad argument");
    cudaSetDevice(h->device);
    Workspace& ws = batched ? h->batchWs : h->ws;
    ws.free_events();
    if (n_ticks == 0) return LVBGS_OK;
    ws.tev.resize((size_t)n_ticks * (kTimedKernels + 1));
    for (cudaEvent_t& e : ws.tev) LV_CUDA(h, cudaEventCreate(&e), "event creation");
    ws.tevTicks = n_ticks;
    return LVBGS_OK;
}

int lvbgs_debug_tick_profile(lvbgs_handle h, int batched, double* out_ms, int max_n) {
    if (!h || !out_ms || max_n <= 0) return 0;
    cudaSetDevice(h->device);
    Workspace& ws = batched ? h->batchWs : h->ws;
    if (ws.tevRecorded == 0) return 0;
    const int n = std::min(max_n, kTimedKernels);
    for (int k = 0; k < n; ++k) out_ms[k] = 0.0;
    for (int t = 0; t < ws.tevRecorded; ++t) {
        cudaEvent_t* ev = &ws.tev[(size_t)t * (kTimedKernels + 1)];
        if (cudaEventSynchronize(ev[kTimedKernels]) != cudaSuccess) return 0;
        for (int k = 0; k < n; ++k) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, ev[k], ev[k + 1]) != cudaSuccess) return 0;
            out_ms[k] += ms;
        }
    }
    for (int k = 0; k < n; ++k) out_ms[k] /= ws.tevRecorded;
    ws.tevRecorded = 0;
    ws.tevNext = 0;
    return n;
}

int lvbgs_debug_repair_phases(lvbgs_handle h, int batched, double* out_us, int max_n) {
    if (!h || !out_us || max_n <= 0) return 0;
    cudaSetDevice(h->device);
    Workspace& ws = batched ? h->batchWs : h->ws;
    if (!ws.work) return 0;
    TickWork w;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) return 0;
    if (cudaMemcpy(&w, ws.work, sizeof(w), cudaMemcpyDeviceToHost) != cudaSuccess) return 0;
    const int n = std::min<int>(max_n, (int)std::min<unsigned>(w.nts, 40u) - 1);
    for (int k = 0; k < n; ++k) out_us[k] = (double)(w.ts[k + 1] - w.ts[k]) / 1e3;
    // then the re-matched items of each round
    int m = std::max(n, 0);
    for (unsigned r = 0; r < std::min(w.iters, 16u) && m < max_n; ++r) out_us[m++] = (double)w.phase_ctr[r];
    return m;
}

lvbgs_status lvbgs_get_scalars(lvbgs_handle h, lvbgs_scalars* out) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (!out) return fail(h, LVBGS_BAD_ARG, "null output");
    if (h->algo == LVBGS_ALGO_LOBSTER || h->algo == LVBGS_ALGO_VIBE || h->algo == LVBGS_ALGO_PBAS) {
        // LOBSTER, ViBe and PBAS keep no frame counter; frame_idx counts their apply() calls
        std::memset(out, 0, sizeof(*out));
        unsigned long long st[2] = {0, 0};
        std::string err;
        s = lob_stats(*h->lob, st, h->stream, err);
        if (s != LVBGS_OK) return fail(h, s, err);
        out->frame_idx = h->lob->frames;
        out->median_blur_kernel_size = h->prm.default_median_blur_kernel_size;
        out->n_relevant_px = h->lob->n_rel;
        out->orig_roi_px = h->lob->orig_roi;
        out->stat_samples_evaluated = st[0];
        out->stat_sample_writes = st[1];
        return LVBGS_OK;
    }
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "sync");
    StreamCtl c;
    LV_CUDA(h, cudaMemcpy(&c, h->sd.ctl, sizeof(c), cudaMemcpyDeviceToHost), "control read");
    std::memset(out, 0, sizeof(*out));
    out->frame_idx = c.frame_idx;
    out->frames_since_last_reset = c.frames_since_reset;
    out->model_reset_cooldown = c.cooldown;
    out->auto_model_reset_enabled = c.auto_reset;
    out->learning_rate_scaling_enabled = c.lr_scaling;
    out->use_3x3_spread = c.use3x3;
    out->median_blur_kernel_size = c.median_k;
    out->lr_lower_cap = c.t_lo;
    out->lr_upper_cap = c.t_hi;
    out->last_nonzero_desc_ratio = c.last_nz_ratio;
    out->nonzero_desc_count = c.last_nz;
    out->tot_color_diff = c.last_colordiff;
    out->n_relevant_px = c.n_rel;
    out->orig_roi_px = c.orig_roi;
    out->stat_samples_evaluated = c.st_samples;
    out->stat_sample_writes = c.st_writes;
    out->stat_repair_rounds = c.st_rounds;
    out->stat_repair_rematched = c.st_rematched;
    return LVBGS_OK;
}

}  // extern "C"

// ---- PAWCS-specific entry points ----
lvbgs_status lvbgs_pawcs_refresh_model(lvbgs_handle h, size_t base_occ, float decr, int force) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (h->algo != LVBGS_ALGO_PAWCS) return fail(h, LVBGS_BAD_ARG, "not a PAWCS handle");
    // BackgroundSubtractorPAWCS.cpp:109-110
    if (!(decr >= 0.0f && decr <= 1.0f))
        return fail(h, LVBGS_BAD_ARG, "model occurrence decrementation must be given as a non-null fraction");
    if (base_occ > 0xffffffffull) return fail(h, LVBGS_UNSUPPORTED, "base occurrence count above 2^32");
    const int buf = (int)(h->pw_frames & 1ull);
    if ((s = pw_upload_desc(h, h->stream)) != LVBGS_OK) return s;
    if ((s = pw_refresh(h, (uint32_t)h->pw_frames, buf, (int)base_occ, decr, force ? 1 : 0, 0, 1, h->stream)) != LVBGS_OK)
        return s;
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "refresh");
    return LVBGS_OK;
}

lvbgs_status lvbgs_pawcs_get_scalars(lvbgs_handle h, lvbgs_pawcs_scalars* out) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    if (h->algo != LVBGS_ALGO_PAWCS || !out) return fail(h, LVBGS_BAD_ARG, "not a PAWCS handle or null output");
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "sync");
    StreamCtl c;
    PawcsCtl pc;
    LV_CUDA(h, cudaMemcpy(&c, h->sd.ctl, sizeof(c), cudaMemcpyDeviceToHost), "control read");
    LV_CUDA(h, cudaMemcpy(&pc, h->pd.pc, sizeof(pc), cudaMemcpyDeviceToHost), "control read");
    std::memset(out, 0, sizeof(*out));
    out->frame_idx = c.frame_idx;
    out->frames_since_last_reset = c.frames_since_reset;
    out->model_reset_cooldown = c.cooldown;
    out->lword_weight_offset = pc.lword_offset;
    out->auto_model_reset_enabled = c.auto_reset;
    out->using_moving_camera = pc.moving_cam;
    out->median_blur_kernel_size = c.median_k;
    out->n_local_words = pc.L;
    out->n_global_words = pc.G;
    out->last_nonflat_ratio = pc.last_nonflat_ratio;
    out->n_relevant_px = c.n_rel;
    out->orig_roi_px = c.orig_roi;
    out->ds_roi_px = pc.ds_roi_count;
    out->fixed_point_rounds = (uint64_t)h->pw_rounds_last;
    return LVBGS_OK;
}

size_t lvbgs_pawcs_debug_export_bytes(lvbgs_handle h, int which) {
    if (!h || h->algo != LVBGS_ALGO_PAWCS || !h->initialized) return 0;
    const size_t npx = h->npx, nw = h->n_rel * (size_t)h->pd.L, gmap = (size_t)h->pd.gwW * h->pd.gwH;
    const size_t nds = (size_t)h->sd.dsW * h->sd.dsH;
    switch (which) {
    case LVBGS_PAWCS_MAP_R: case LVBGS_PAWCS_MAP_V: case LVBGS_PAWCS_MAP_T: case LVBGS_PAWCS_MAP_DMIN_LT:
    case LVBGS_PAWCS_MAP_DMIN_ST: case LVBGS_PAWCS_MAP_RAW_LT: case LVBGS_PAWCS_MAP_RAW_ST:
    case LVBGS_PAWCS_MAP_FIN_LT: case LVBGS_PAWCS_MAP_FIN_ST: return npx * 4;
    case LVBGS_PAWCS_MAP_ILLUM: case LVBGS_PAWCS_MAP_UNSTABLE: case LVBGS_PAWCS_MAP_BLINKS:
    case LVBGS_PAWCS_MAP_LAST_RAW_FG: case LVBGS_PAWCS_MAP_LAST_FG: case LVBGS_PAWCS_MAP_LAST_FG_DIL:
    case LVBGS_PAWCS_MAP_LAST_RAW_BLINK: case LVBGS_PAWCS_MAP_ROI: return npx;
    case LVBGS_PAWCS_MAP_LAST_COLOR: return npx * h->C;
    case LVBGS_PAWCS_MAP_LAST_DESC: return npx * 2 * h->C;
    case LVBGS_PAWCS_MAP_DS_LT: case LVBGS_PAWCS_MAP_DS_ST: return nds * 4 * h->C;
    case LVBGS_PAWCS_MAP_LUT: return 256;
    case LVBGS_PAWCS_MAP_LW_COLOR: return nw * h->C;
    case LVBGS_PAWCS_MAP_LW_DESC: return nw * 2 * h->C;
    case LVBGS_PAWCS_MAP_LW_OCC: case LVBGS_PAWCS_MAP_LW_FIRST: case LVBGS_PAWCS_MAP_LW_LAST: return nw * 8;
    case LVBGS_PAWCS_MAP_GW: return (size_t)h->pd.G * 20;
    case LVBGS_PAWCS_MAP_GW_MAP: return (size_t)h->pd.G * gmap * 4;
    case LVBGS_PAWCS_MAP_GLUT: return npx * (size_t)h->pd.G;
    default: return 0;
    }
}

lvbgs_status lvbgs_pawcs_debug_export(lvbgs_handle h, int which, void* out, size_t bytes) {
    lvbgs_status s = check_ready(h);
    if (s != LVBGS_OK) return s;
    const size_t need = lvbgs_pawcs_debug_export_bytes(h, which);
    if (!need || !out || bytes < need) return fail(h, LVBGS_BAD_ARG, "unknown map or output too small");
    LV_CUDA(h, cudaStreamSynchronize(h->stream), "sync");
    const size_t npx = h->npx, L = (size_t)h->pd.L, G = (size_t)h->pd.G;
    const size_t gmap = (size_t)h->pd.gwW * h->pd.gwH, nds = (size_t)h->sd.dsW * h->sd.dsH;
    const int buf = (int)(h->pw_frames & 1ull);
    auto dl = [&](void* dst, const void* src, size_t n) { return cudaMemcpy(dst, src, n, cudaMemcpyDeviceToHost); };
    const float* fm = h->sd.fm + (size_t)buf * kNumFloatMaps * npx;
    int fmap = -1;
    switch (which) {
    case LVBGS_PAWCS_MAP_R: fmap = FM_R; break;
    case LVBGS_PAWCS_MAP_V: fmap = FM_V; break;
    case LVBGS_PAWCS_MAP_T: fmap = FM_T; break;
    case LVBGS_PAWCS_MAP_DMIN_LT: fmap = FM_DMIN_LT; break;
    case LVBGS_PAWCS_MAP_DMIN_ST: fmap = FM_DMIN_ST; break;
    case LVBGS_PAWCS_MAP_RAW_LT: fmap = FM_RAW_LT; break;
    case LVBGS_PAWCS_MAP_RAW_ST: fmap = FM_RAW_ST; break;
    case LVBGS_PAWCS_MAP_FIN_LT: fmap = FM_FIN_LT; break;
    case LVBGS_PAWCS_MAP_FIN_ST: fmap = FM_FIN_ST; break;
    default: break;
    }
    cudaError_t e = cudaSuccess;
    if (fmap >= 0) {
        e = dl(out, fm + (size_t)fmap * npx, npx * 4);
    } else {
        switch (which) {
        case LVBGS_PAWCS_MAP_ILLUM: e = dl(out, h->pd.illum, npx); break;
        case LVBGS_PAWCS_MAP_UNSTABLE: e = dl(out, h->pd.unstable, npx); break;
        case LVBGS_PAWCS_MAP_BLINKS: e = dl(out, h->sd.blinks, npx); break;
        case LVBGS_PAWCS_MAP_LAST_RAW_FG: e = dl(out, h->sd.lastRawFG, npx); break;
        case LVBGS_PAWCS_MAP_LAST_FG: e = dl(out, h->sd.lastFG, npx); break;
        case LVBGS_PAWCS_MAP_LAST_FG_DIL: {
            // stored inverted; before the first frame the dilated mask is all clear
            e = dl(out, h->sd.dilInv, npx);
            uint8_t* o = (uint8_t*)out;
            for (size_t i = 0; i < npx; ++i) o[i] = h->pw_frames ? (uint8_t)~o[i] : 0;
            break;
        }
        case LVBGS_PAWCS_MAP_LAST_RAW_BLINK: e = dl(out, h->sd.lastRawBlink, npx); break;
        case LVBGS_PAWCS_MAP_ROI: e = dl(out, h->sd.roi, npx); break;
        case LVBGS_PAWCS_MAP_LAST_COLOR: e = dl(out, h->sd.lastCol, npx * h->C); break;
        case LVBGS_PAWCS_MAP_LAST_DESC: e = dl(out, h->sd.lastDesc, npx * 2 * h->C); break;
        case LVBGS_PAWCS_MAP_DS_LT: e = dl(out, h->sd.dsLT, nds * 4 * h->C); break;
        case LVBGS_PAWCS_MAP_DS_ST: e = dl(out, h->sd.dsST, nds * 4 * h->C); break;
        case LVBGS_PAWCS_MAP_LUT: {
            StreamCtl c;
            e = dl(&c, h->sd.ctl, sizeof(c));
            std::memcpy(out, c.lut, 256);
            break;
        }
        case LVBGS_PAWCS_MAP_GW_MAP: e = dl(out, h->pd.gmap, G * gmap * 4); break;
        case LVBGS_PAWCS_MAP_GLUT: {
            std::vector<uint8_t> g(npx * kPwGlutStride);
            e = dl(g.data(), h->pd.glut, npx * kPwGlutStride);
            uint8_t* o = (uint8_t*)out;
            for (size_t i = 0; i < npx; ++i)
                for (size_t k = 0; k < G; ++k) o[i * G + k] = h->roi[i] ? g[i * kPwGlutStride + k] : 0;
            break;
        }
        case LVBGS_PAWCS_MAP_GW: {
            PawcsCtl pc;
            e = dl(&pc, h->pd.pc, sizeof(pc));
            uint8_t* b = (uint8_t*)out;
            std::memset(b, 0, G * 20);
            for (size_t w = 0; w < G; ++w) {
                uint8_t* r = b + w * 20;
                const uint16_t d[3] = {(uint16_t)pc.gw_desc[w], (uint16_t)(pc.gw_desc[w] >> 16), (uint16_t)pc.gw_desc2[w]};
                for (int c = 0; c < h->C; ++c) {
                    r[c] = (uint8_t)(pc.gw_color[w] >> (8 * c));
                    std::memcpy(r + 4 + 2 * c, &d[c], 2);
                }
                r[10] = (uint8_t)pc.gw_bits[w];
                std::memcpy(r + 12, &pc.gw_weight[w], 4);
                int32_t slot = -1;
                for (size_t g = 0; g < G; ++g)
                    if (pc.gdict[g] == (int)w) slot = (int32_t)g;
                std::memcpy(r + 16, &slot, 4);
            }
            break;
        }
        case LVBGS_PAWCS_MAP_LW_COLOR: case LVBGS_PAWCS_MAP_LW_DESC: case LVBGS_PAWCS_MAP_LW_OCC:
        case LVBGS_PAWCS_MAP_LW_FIRST: case LVBGS_PAWCS_MAP_LW_LAST: {
            // model-major (ROI pixels in raster order), slot-minor, as the reference's dictionary
            const size_t es = which == LVBGS_PAWCS_MAP_LW_COLOR  ? (size_t)h->C
                              : which == LVBGS_PAWCS_MAP_LW_DESC ? 2 * (size_t)h->C
                                                                 : 4;
            const void* src = which == LVBGS_PAWCS_MAP_LW_COLOR  ? (const void*)h->pd.wColor
                              : which == LVBGS_PAWCS_MAP_LW_DESC ? (const void*)h->pd.wDesc
                              : which == LVBGS_PAWCS_MAP_LW_OCC  ? (const void*)h->pd.wOcc
                              : which == LVBGS_PAWCS_MAP_LW_FIRST ? (const void*)h->pd.wFirst
                                                                  : (const void*)h->pd.wLast;
            std::vector<uint8_t> planes(L * npx * es);
            e = dl(planes.data(), (const uint8_t*)src + (size_t)buf * L * npx * es, planes.size());
            size_t m = 0;
            for (size_t i = 0; i < npx; ++i) {
                if (!h->roi[i]) continue;
                for (size_t j = 0; j < L; ++j) {
                    const size_t k = m * L + j;
                    const uint8_t* v = planes.data() + (j * npx + i) * es;
                    if (es == 4) {
                        uint32_t u;
                        std::memcpy(&u, v, 4);
                        const uint64_t u64 = u;
                        std::memcpy((uint8_t*)out + k * 8, &u64, 8);
                    } else {
                        std::memcpy((uint8_t*)out + k * es, v, es);
                    }
                }
                ++m;
            }
            break;
        }
        default: return fail(h, LVBGS_BAD_ARG, "unknown map");
        }
    }
    if (e != cudaSuccess) return cuda_fail(h, e, "map download");
    return LVBGS_OK;
}
