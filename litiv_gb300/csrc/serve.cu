// Serving loop over the lvbgs C-ABI (include/lvserve.h): admission by device bytes, continuous
// batching of the frames that arrive while ticks run, spill of idle streams to pinned host memory,
// and the serving workload simulator (Poisson stream arrivals, 30 fps per stream).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lvbgs.h"
#include "../../include/lvbgs_synth.h"
#include "../../include/lvserve.h"

namespace {

using Clock = std::chrono::steady_clock;
double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

// latencies kept for the quantiles (the most recent ones)
constexpr size_t kLatCap = 1u << 22;
// share of the batch work area per resident pixel (four repair lists of 64-bit entries)
constexpr size_t kWorkBytesPerPx = 4 * sizeof(unsigned long long);

struct Req {
    const uint8_t* img;
    size_t stride;
    uint8_t* mask;
    double lr;
    uint64_t tag;
    Clock::time_point t0;
};

// S_INIT: a PAWCS stream admitted (its bytes reserved) whose handle a PAWCS lane is creating;
// reported as S_WAITING
enum { S_RESIDENT = 0, S_WAITING = 1, S_SPILLED = 2, S_CLOSED = 3, S_INIT = 4 };

struct SStream {
    int id = 0;
    lvbgs_algo algo = LVBGS_ALGO_SUBSENSE;
    lvbgs_params prm{};
    int W = 0, H = 0, C = 0;
    std::vector<uint8_t> init, roi;
    int state = S_WAITING;
    lvbgs_handle h = nullptr;
    std::deque<Req> q;
    bool inFlight = false, closing = false, failed = false;
    bool laneDestroy = false;  // PAWCS: a lane destroys the handle (freeing memory waits for the device)
    size_t bytes = 0;       // accounted device bytes while resident
    size_t stateBytes = 0;  // size of the spill image
    void* spill = nullptr;
    size_t spillCap = 0;
    Clock::time_point lastActive, tOpen, tClosed;
    size_t npx() const { return (size_t)W * H; }
};

struct Tick {
    uint64_t ticket = 0;
    std::vector<SStream*> ss;
    std::vector<Req> reqs;
};

}  // namespace

struct lvserve_ctx {
    lvserve_config cfg{};
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::thread th;
    std::vector<std::thread> lanes;  // PAWCS lanes
    bool stop = false;
    std::map<int, std::unique_ptr<SStream>> streams;
    std::deque<SStream*> admitQ;
    std::deque<lvserve_result> results;
    size_t maxResults = 1 << 20;
    std::vector<double> lat;  // latencies of finished frames, a ring of kLatCap
    size_t latPos = 0;
    lvserve_stats st{};
    double tickStreamsSum = 0;
    int nextId = 1;
    int queued = 0;    // frames queued, not yet in a tick
    int inflightN = 0; // ticks in flight
    std::string err;
    // simulator hooks, called with mu held
    std::function<void(const SStream&, const Req&, Clock::time_point, int)> onDone;
    std::function<void(const SStream&, Clock::time_point)> onAdmit;
    // owned by the scheduler thread
    lvbgs_batch batch = nullptr;
    cudaStream_t stream = nullptr;
    std::deque<Tick> inflight;
    size_t used = 0;  // accounted device bytes of resident streams
    size_t hostSpilled = 0;
    size_t reservedPx = 0;
    int reservedStreams = 0;
    Clock::time_point busySince;
    std::multimap<size_t, void*> pinnedFree;  // spill buffers kept for reuse
};

namespace {

void set_err(lvserve_ctx* s, const std::string& m) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = m;
}

void* take_pinned(lvserve_ctx* s, size_t bytes, size_t* cap) {
    auto it = s->pinnedFree.lower_bound(bytes);
    if (it != s->pinnedFree.end() && it->first <= bytes + bytes / 4) {
        void* p = it->second;
        *cap = it->first;
        s->pinnedFree.erase(it);
        return p;
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    *cap = bytes;
    return p;
}

// completes the ticks in flight that have finished (the oldest first; `block`: wait for the oldest)
void retire(lvserve_ctx* s, bool block) {
    while (!s->inflight.empty()) {
        Tick& t = s->inflight.front();
        if (!block && lvbgs_batch_query(s->batch, t.ticket) == 0) break;
        block = false;
        const lvbgs_status r = lvbgs_batch_complete(s->batch, t.ticket);
        const Clock::time_point now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (r != LVBGS_OK && s->err.empty()) s->err = lvbgs_last_error(nullptr);
            for (size_t i = 0; i < t.ss.size(); ++i) {
                SStream* x = t.ss[i];
                x->inFlight = false;
                x->lastActive = now;
                if (r != LVBGS_OK) x->failed = true;
                const double l = ms_between(t.reqs[i].t0, now);
                if (s->lat.size() < kLatCap) s->lat.push_back(l);
                else s->lat[s->latPos++ % kLatCap] = l;
                if (s->results.size() < s->maxResults) s->results.push_back({x->id, t.reqs[i].tag, (int)r, l});
                ++s->st.frames_done;
                s->st.px_done += x->npx();
                if (s->onDone) s->onDone(*x, t.reqs[i], now, (int)r);
            }
            --s->inflightN;
            if (s->inflightN == 0) s->st.busy_ms += ms_between(s->busySince, now);
        }
        s->inflight.pop_front();
        s->cvDone.notify_all();
    }
}

// room planning: the longest-idle eligible candidates first, nothing chosen unless the need fits
int plan_room(size_t used, size_t budget, size_t need, const size_t* bytes, const double* idle, int n, double minIdle,
              int* out) {
    if (used + need <= budget) return 0;
    if (need > budget) return -1;
    std::vector<int> order;
    for (int i = 0; i < n; ++i)
        if (idle[i] >= minIdle) order.push_back(i);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return idle[a] > idle[b]; });
    size_t u = used;
    int k = 0;
    for (int i : order) {
        if (u + need <= budget) break;
        u -= std::min(u, bytes[i]);
        out[k++] = i;
    }
    return (u + need <= budget) ? k : -1;
}

bool spill_stream(lvserve_ctx* s, SStream* x) {
    const bool lane = x->algo == LVBGS_ALGO_PAWCS;
    if (lane) {
        // PAWCS frames run on the lanes: claim the stream as a lane claims a frame, so that no lane
        // starts one of its frames while its state is copied out
        std::lock_guard<std::mutex> lk(s->mu);
        if (x->state != S_RESIDENT || x->inFlight || !x->q.empty()) return false;
        x->inFlight = true;
    }
    auto release = [&] {
        if (!lane) return;
        std::lock_guard<std::mutex> lk(s->mu);
        x->inFlight = false;
    };
    size_t cap = 0;
    void* buf = x->spill ? x->spill : take_pinned(s, x->stateBytes, &cap);
    if (!buf) {
        release();
        return false;
    }
    if (!x->spill) x->spillCap = cap;
    x->spill = buf;
    if (lvbgs_spill(x->h, buf, x->spillCap) != LVBGS_OK) {
        set_err(s, lvbgs_last_error(x->h));
        release();
        return false;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    if (lane) x->inFlight = false;
    x->state = S_SPILLED;
    s->used -= x->bytes;
    s->hostSpilled += x->stateBytes;
    ++s->st.spills;
    return true;
}

// makes room for `need` bytes by spilling idle resident streams (none chosen if it cannot fit)
bool make_room(lvserve_ctx* s, size_t need, const SStream* except) {
    std::vector<SStream*> cand;
    std::vector<size_t> bytes;
    std::vector<double> idle;
    size_t used, budget = s->cfg.hbm_budget_bytes;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        used = s->used;
        if (used + need <= budget) return true;
        const Clock::time_point now = Clock::now();
        for (auto& kv : s->streams) {
            SStream* x = kv.second.get();
            if (x == except || x->state != S_RESIDENT || x->inFlight || !x->q.empty()) continue;
            if (s->cfg.host_spill_budget_bytes && s->hostSpilled + x->stateBytes > s->cfg.host_spill_budget_bytes)
                continue;
            cand.push_back(x);
            bytes.push_back(x->bytes);
            idle.push_back(ms_between(x->lastActive, now));
        }
    }
    std::vector<int> pick(cand.size());
    const int k = plan_room(used, budget, need, bytes.data(), idle.data(), (int)cand.size(), s->cfg.idle_spill_ms,
                            pick.data());
    if (k < 0) return false;
    size_t spilledHost = 0;
    for (int i = 0; i < k; ++i) spilledHost += cand[pick[i]]->stateBytes;
    if (s->cfg.host_spill_budget_bytes && s->hostSpilled + spilledHost > s->cfg.host_spill_budget_bytes) return false;
    for (int i = 0; i < k; ++i)
        if (!spill_stream(s, cand[pick[i]])) return false;
    return true;
}

void fail_queue(lvserve_ctx* s, SStream* x, int status) {
    // frames of a stream that cannot run are returned with the error (mu held)
    const Clock::time_point now = Clock::now();
    while (!x->q.empty()) {
        const Req r = x->q.front();
        x->q.pop_front();
        --s->queued;
        const double l = ms_between(r.t0, now);
        if (s->results.size() < s->maxResults) s->results.push_back({x->id, r.tag, status, l});
        if (s->onDone) s->onDone(*x, r, now, status);
    }
}

void destroy_stream(lvserve_ctx* s, SStream* x) {
    if (x->h) lvbgs_destroy(x->h);
    x->h = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    if ((x->state == S_RESIDENT || x->state == S_INIT) && x->bytes) s->used -= x->bytes;
    if (x->state == S_SPILLED) s->hostSpilled -= x->stateBytes;
    if (x->spill) s->pinnedFree.emplace(x->spillCap, x->spill);
    x->spill = nullptr;
    if (x->state == S_WAITING) {
        auto it = std::find(s->admitQ.begin(), s->admitQ.end(), x);
        if (it != s->admitQ.end()) s->admitQ.erase(it);
    }
    x->state = S_CLOSED;
    ++s->st.closed;
    s->streams.erase(x->id);
    s->cvDone.notify_all();
}

// closes, restores and admissions, in that order
void housekeeping(lvserve_ctx* s) {
    std::vector<SStream*> closing, restore;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto& kv : s->streams) {
            SStream* x = kv.second.get();
            if (s->stop && x->state == S_WAITING) fail_queue(s, x, LVBGS_BUSY);  // shutting down: no admission
            if (x->closing && x->q.empty() && !x->inFlight) {
                // PAWCS handles are destroyed on a PAWCS lane, so that the device-wide wait of freeing
                // their memory does not hold the ticks back
                // (a PAWCS stream still waiting for its handle, S_INIT, is left to the lanes)
                if (x->algo == LVBGS_ALGO_PAWCS && x->h) x->laneDestroy = true;
                else if (!(x->algo == LVBGS_ALGO_PAWCS && x->state == S_INIT)) closing.push_back(x);
            } else if (x->state == S_SPILLED && !x->q.empty()) {
                restore.push_back(x);
            }
        }
        std::sort(restore.begin(), restore.end(),
                  [](const SStream* a, const SStream* b) { return a->q.front().t0 < b->q.front().t0; });
    }
    // a handle's destruction frees device memory, which waits for the device: defer it while
    // ticks are in flight, unless the stream was closed long ago
    const Clock::time_point now = Clock::now();
    for (SStream* x : closing) {
        if (x->h && !s->inflight.empty() && ms_between(x->tClosed, now) < 250.0) continue;
        destroy_stream(s, x);
    }
    for (SStream* x : restore) {
        if (!make_room(s, x->bytes, x)) break;
        if (lvbgs_restore(x->h, x->spill, x->spillCap) != LVBGS_OK) {
            set_err(s, lvbgs_last_error(x->h));
            std::lock_guard<std::mutex> lk(s->mu);
            x->failed = true;
            fail_queue(s, x, LVBGS_DEVICE_ERROR);
            continue;
        }
        std::lock_guard<std::mutex> lk(s->mu);
        x->state = S_RESIDENT;
        s->used += x->bytes;
        s->hostSpilled -= x->stateBytes;
        x->lastActive = Clock::now();
        ++s->st.restores;
    }
    for (;;) {
        SStream* x = nullptr;
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (s->admitQ.empty()) break;
            x = s->admitQ.front();
        }
        if (!make_room(s, x->bytes, x)) break;  // first come, first served
        if (x->algo == LVBGS_ALGO_PAWCS) {
            // created and initialized on a PAWCS lane: refreshModel over every pixel (tens of ms for a
            // 1080p BGR stream) would hold the ticks back
            std::lock_guard<std::mutex> lk(s->mu);
            s->admitQ.pop_front();
            x->state = S_INIT;
            s->used += x->bytes;
            s->st.peak_device_bytes = std::max(s->st.peak_device_bytes, s->used);
            s->cvWork.notify_all();
            continue;
        }
        lvbgs_handle h = nullptr;
        lvbgs_status r = lvbgs_create(x->algo, &x->prm, &h);
        if (r == LVBGS_OK)
            r = lvbgs_initialize(h, x->init.data(), x->W, x->H, x->C, 0, x->roi.empty() ? nullptr : x->roi.data());
        std::lock_guard<std::mutex> lk(s->mu);
        s->admitQ.pop_front();
        if (r != LVBGS_OK) {
            s->err = lvbgs_last_error(h);
            if (h) lvbgs_destroy(h);
            x->failed = true;
            x->state = S_CLOSED;
            fail_queue(s, x, r);
            x->closing = true;
            continue;
        }
        x->h = h;
        x->state = S_RESIDENT;
        x->init.clear();
        x->init.shrink_to_fit();
        x->lastActive = Clock::now();
        s->used += x->bytes;
        s->st.peak_device_bytes = std::max(s->st.peak_device_bytes, s->used);
        ++s->st.admitted;
        if (s->onAdmit) s->onAdmit(*x, x->lastActive);
    }
}

// launches one tick over the resident streams with a queued frame and none in flight
bool launch(lvserve_ctx* s, std::vector<lvbgs_handle>& hs, std::vector<lvbgs_frame>& fr) {
    Tick t;
    size_t px = 0;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        for (auto& kv : s->streams) {
            SStream* x = kv.second.get();
            if (x->algo != LVBGS_ALGO_SUBSENSE) continue;  // PAWCS streams run on the PAWCS lanes
            if (x->state != S_RESIDENT || x->inFlight || x->q.empty() || x->failed) continue;
            t.ss.push_back(x);
            px += x->npx();
        }
    }
    if (t.ss.empty()) return false;
    if (px > s->reservedPx || (int)t.ss.size() > s->reservedStreams) {
        if (s->inflight.empty()) {
            // grow the work area with headroom (only while nothing is in flight)
            const size_t npx = std::max(px, s->reservedPx + s->reservedPx / 2);
            const int ns = std::max((int)t.ss.size(), s->reservedStreams + s->reservedStreams / 2);
            if (lvbgs_batch_reserve(s->batch, npx, ns) == LVBGS_OK) {
                s->reservedPx = npx;
                s->reservedStreams = ns;
            }
        }
        // take the streams that fit the current work area; the others join a later tick
        size_t acc = 0;
        size_t k = 0;
        while (k < t.ss.size() && (int)k < s->reservedStreams && acc + t.ss[k]->npx() <= s->reservedPx)
            acc += t.ss[k++]->npx();
        if (k == 0) return false;
        t.ss.resize(k);
    }
    hs.clear();
    fr.clear();
    {
        // the tick counts as in flight from here, so that a drain never sees its frames nowhere
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->inflightN == 0) s->busySince = Clock::now();
        ++s->inflightN;
        for (SStream* x : t.ss) {
            const Req r = x->q.front();
            x->q.pop_front();
            --s->queued;
            x->inFlight = true;
            t.reqs.push_back(r);
            hs.push_back(x->h);
            fr.push_back(lvbgs_frame{r.img, r.stride, r.mask, r.lr});
        }
    }
    const lvbgs_status r = lvbgs_batch_submit(s->batch, hs.data(), fr.data(), (int)hs.size(), s->stream, &t.ticket);
    const Clock::time_point now = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    if (r != LVBGS_OK) {
        if (s->err.empty()) s->err = lvbgs_last_error(hs[0]);
        --s->inflightN;
        if (s->inflightN == 0) s->st.busy_ms += ms_between(s->busySince, now);
        for (size_t i = 0; i < t.ss.size(); ++i) {
            SStream* x = t.ss[i];
            x->inFlight = false;
            x->failed = true;
            if (s->results.size() < s->maxResults) s->results.push_back({x->id, t.reqs[i].tag, (int)r, 0.0});
            if (s->onDone) s->onDone(*x, t.reqs[i], now, (int)r);
            fail_queue(s, x, (int)r);
        }
        s->cvDone.notify_all();
        return false;
    }
    ++s->st.ticks;
    s->tickStreamsSum += (double)t.ss.size();
    s->inflight.push_back(std::move(t));
    return true;
}

// A PAWCS lane: PAWCS frame steps wait on the host for their fixed-point rounds, so they cannot join
// a batched tick; each lane takes the oldest queued frame of a resident PAWCS stream and runs it on
// that stream's own CUDA stream, beside the batched SuBSENSE ticks. A stream's frames run in
// submission order (one in flight per stream), so its results are those of the stream alone.
void pawcs_lane(lvserve_ctx* s) {
    cudaSetDevice(s->cfg.device_id);
    // the lane's frames run on a stream of the lowest priority: when the blocks of a PAWCS kernel
    // drain, the ticks' pending blocks (highest priority) are scheduled first, so a PAWCS stream
    // that costs more than the device can give (a 1080p BGR stream at 30 fps) queues its own frames
    // instead of delaying the batched ones
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    cudaStream_t lst = nullptr;
    if (cudaStreamCreateWithPriority(&lst, cudaStreamNonBlocking, least) != cudaSuccess) {
        cudaGetLastError();
        lst = nullptr;  // the handle's own stream
    }
    for (;;) {
        SStream* x = nullptr;
        Req r;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            // handle destruction and creation first (claimed with inFlight)
            SStream* job = nullptr;
            for (auto& kv : s->streams) {
                SStream* y = kv.second.get();
                if (y->algo != LVBGS_ALGO_PAWCS || y->inFlight) continue;
                // an admitted stream waiting for its handle is set up also when it was closed meanwhile
                // (its queued frames still run; with none queued it just goes)
                if (y->laneDestroy || y->state == S_INIT) {
                    job = y;
                    break;
                }
            }
            if (job) {
                job->inFlight = true;
                const bool drop = job->laneDestroy || (job->closing && job->q.empty());
                lk.unlock();
                if (drop) {
                    destroy_stream(s, job);
                } else {
                    lvbgs_handle h = nullptr;
                    lvbgs_status rc = lvbgs_create(job->algo, &job->prm, &h);
                    if (rc == LVBGS_OK)
                        rc = lvbgs_initialize(h, job->init.data(), job->W, job->H, job->C, 0,
                                              job->roi.empty() ? nullptr : job->roi.data());
                    std::lock_guard<std::mutex> lk2(s->mu);
                    job->inFlight = false;
                    if (rc != LVBGS_OK) {
                        s->err = lvbgs_last_error(h);
                        if (h) lvbgs_destroy(h);
                        s->used -= job->bytes;
                        job->failed = true;
                        job->state = S_CLOSED;
                        fail_queue(s, job, rc);
                        job->closing = true;
                    } else {
                        job->h = h;
                        job->state = S_RESIDENT;
                        job->init.clear();
                        job->init.shrink_to_fit();
                        job->lastActive = Clock::now();
                        ++s->st.admitted;
                        if (s->onAdmit) s->onAdmit(*job, job->lastActive);
                    }
                }
                s->cvDone.notify_all();
                s->cvWork.notify_all();
                continue;
            }
            for (auto& kv : s->streams) {
                SStream* y = kv.second.get();
                if (y->algo != LVBGS_ALGO_PAWCS || y->state != S_RESIDENT || y->inFlight || y->q.empty() || y->failed)
                    continue;
                if (!x || y->q.front().t0 < x->q.front().t0) x = y;
            }
            if (!x) {
                if (s->stop && s->streams.empty()) break;
                s->cvWork.wait_for(lk, std::chrono::microseconds(1000));
                continue;
            }
            r = x->q.front();
            x->q.pop_front();
            --s->queued;
            x->inFlight = true;
            if (s->inflightN == 0) s->busySince = Clock::now();
            ++s->inflightN;
        }
        const lvbgs_status st = lvbgs_apply(x->h, r.img, r.stride, r.mask, r.lr, lst);
        const Clock::time_point now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(s->mu);
            if (st != LVBGS_OK && s->err.empty()) s->err = lvbgs_last_error(x->h);
            x->inFlight = false;
            x->lastActive = now;
            const double l = ms_between(r.t0, now);
            if (s->lat.size() < kLatCap) s->lat.push_back(l);
            else s->lat[s->latPos++ % kLatCap] = l;
            if (s->results.size() < s->maxResults) s->results.push_back({x->id, r.tag, (int)st, l});
            ++s->st.frames_done;
            s->st.px_done += x->npx();
            ++s->st.pawcs_frames;
            if (s->onDone) s->onDone(*x, r, now, (int)st);
            if (st != LVBGS_OK) {
                x->failed = true;
                fail_queue(s, x, (int)st);
            }
            --s->inflightN;
            if (s->inflightN == 0) s->st.busy_ms += ms_between(s->busySince, now);
        }
        s->cvDone.notify_all();
        s->cvWork.notify_all();
    }
    if (lst) {
        cudaStreamSynchronize(lst);
        cudaStreamDestroy(lst);
    }
}

void scheduler(lvserve_ctx* s) {
    cudaSetDevice(s->cfg.device_id);
    std::vector<lvbgs_handle> hs;
    std::vector<lvbgs_frame> fr;
    for (;;) {
        retire(s, (int)s->inflight.size() >= s->cfg.max_inflight);
        housekeeping(s);
        bool launched = false;
        if ((int)s->inflight.size() < s->cfg.max_inflight) launched = launch(s, hs, fr);
        std::unique_lock<std::mutex> lk(s->mu);
        if (s->stop && s->streams.empty() && s->inflight.empty()) break;
        if (launched) continue;
        // wake on new work, or poll the oldest tick in flight
        const auto wait = s->inflight.empty() ? std::chrono::microseconds(2000) : std::chrono::microseconds(50);
        s->cvWork.wait_for(lk, wait);
    }
}

}  // namespace

extern "C" {

lvbgs_status lvserve_default_config(lvserve_config* out) {
    if (!out) return LVBGS_BAD_ARG;
    *out = lvserve_config{0, 0, 0, 256, 8, 500.0, 2, 1};
    return LVBGS_OK;
}

lvbgs_status lvserve_create(const lvserve_config* cfg, lvserve_handle* out) {
    if (!out) return LVBGS_BAD_ARG;
    *out = nullptr;
    lvserve_config c;
    lvserve_default_config(&c);
    if (cfg) c = *cfg;
    if (c.max_live <= 0 || c.max_queue <= 0 || c.max_inflight < 1 || c.max_inflight > LVBGS_BATCH_MAX_INFLIGHT ||
        c.idle_spill_ms < 0 || c.pawcs_lanes < 0 || c.pawcs_lanes > 64)
        return LVBGS_BAD_ARG;
    if (cudaSetDevice(c.device_id) != cudaSuccess) return LVBGS_DEVICE_ERROR;
    if (c.hbm_budget_bytes == 0) {
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) return LVBGS_DEVICE_ERROR;
        c.hbm_budget_bytes = fr / 10 * 8;
    }
    std::unique_ptr<lvserve_ctx> s(new lvserve_ctx());
    s->cfg = c;
    s->reservedPx = 1 << 20;
    s->reservedStreams = 64;
    if (lvbgs_batch_create(c.device_id, s->reservedPx, s->reservedStreams, &s->batch) != LVBGS_OK)
        return LVBGS_OOM;
    // with PAWCS lanes, the ticks share the device: the cooperative repair grid takes half of the
    // co-resident blocks so that it can start beside the lanes' kernels
    if (c.pawcs_lanes > 0) lvbgs_batch_set_repair_share(s->batch, 2);
    // the ticks run on a stream of the highest priority (the PAWCS lanes on the lowest)
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (cudaStreamCreateWithPriority(&s->stream, cudaStreamNonBlocking, greatest) != cudaSuccess) {
        lvbgs_batch_destroy(s->batch);
        return LVBGS_DEVICE_ERROR;
    }
    s->th = std::thread(scheduler, s.get());
    for (int i = 0; i < c.pawcs_lanes; ++i) s->lanes.emplace_back(pawcs_lane, s.get());
    *out = s.release();
    return LVBGS_OK;
}

lvbgs_status lvserve_destroy(lvserve_handle s) {
    if (!s) return LVBGS_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        for (auto& kv : s->streams) {
            kv.second->closing = true;
            kv.second->tClosed = Clock::time_point();
        }
        s->cvWork.notify_all();
    }
    s->th.join();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->cvWork.notify_all();
    }
    for (std::thread& t : s->lanes) t.join();
    lvbgs_batch_destroy(s->batch);
    cudaStreamDestroy(s->stream);
    for (auto& kv : s->pinnedFree) cudaFreeHost(kv.second);
    delete s;
    return LVBGS_OK;
}

lvbgs_status lvserve_open(lvserve_handle s, lvbgs_algo algo, const lvbgs_params* params, const uint8_t* img, int W,
                          int H, int C, size_t stride, const uint8_t* roi, int* id) {
    if (!s || !img || !id || W <= 0 || H <= 0) return LVBGS_BAD_ARG;
    if (C != 1 && C != 3) return LVBGS_BAD_TYPE;
    if (algo == LVBGS_ALGO_PAWCS && s->cfg.pawcs_lanes == 0) {
        std::lock_guard<std::mutex> lk(s->mu);
        s->err = "PAWCS streams need pawcs_lanes > 0";
        return LVBGS_UNSUPPORTED;
    }
    const size_t dev = lvbgs_device_bytes(algo, W, H, C, params ? params->bg_samples : 50);
    if (dev == 0) return LVBGS_UNSUPPORTED;
    std::unique_ptr<SStream> x(new SStream());
    x->algo = algo;
    if (params) x->prm = *params;
    else lvbgs_default_params(algo, &x->prm);
    x->prm.device_id = s->cfg.device_id;
    x->W = W;
    x->H = H;
    x->C = C;
    x->bytes = dev + kWorkBytesPerPx * (size_t)W * H;
    x->stateBytes = lvbgs_state_bytes(algo, W, H, C, x->prm.bg_samples);
    const size_t row = (size_t)W * C;
    if (stride == 0) stride = row;
    if (stride < row) return LVBGS_BAD_ARG;
    x->init.resize(row * H);
    for (int y = 0; y < H; ++y) std::memcpy(&x->init[(size_t)y * row], img + (size_t)y * stride, row);
    if (roi) x->roi.assign(roi, roi + (size_t)W * H);
    std::lock_guard<std::mutex> lk(s->mu);
    if (x->bytes > s->cfg.hbm_budget_bytes) {
        s->err = "stream alone exceeds the HBM budget";
        return LVBGS_BAD_SIZE;
    }
    if ((int)s->streams.size() >= s->cfg.max_live) {
        ++s->st.rejected;
        s->err = "server is at max_live streams";
        return LVBGS_BUSY;
    }
    x->id = s->nextId++;
    x->tOpen = Clock::now();
    x->lastActive = x->tOpen;
    SStream* p = x.get();
    s->streams.emplace(p->id, std::move(x));
    s->admitQ.push_back(p);
    *id = p->id;
    s->cvWork.notify_all();
    return LVBGS_OK;
}

lvbgs_status lvserve_submit(lvserve_handle s, int id, const uint8_t* img, size_t stride, uint8_t* mask, double lr,
                            uint64_t tag) {
    if (!s || !img) return LVBGS_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->streams.find(id);
    if (it == s->streams.end() || it->second->closing) {
        s->err = "unknown or closed stream";
        return LVBGS_BAD_ARG;
    }
    SStream* x = it->second.get();
    if (x->failed) {
        s->err = "stream failed earlier";
        return LVBGS_DEVICE_ERROR;
    }
    if ((int)x->q.size() >= s->cfg.max_queue) {
        ++s->st.busy_refusals;
        return LVBGS_BUSY;
    }
    x->q.push_back(Req{img, stride, mask, lr, tag, Clock::now()});
    ++s->queued;
    s->cvWork.notify_all();
    return LVBGS_OK;
}

lvbgs_status lvserve_close(lvserve_handle s, int id) {
    if (!s) return LVBGS_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->streams.find(id);
    if (it == s->streams.end()) return LVBGS_BAD_ARG;
    it->second->closing = true;
    it->second->tClosed = Clock::now();
    s->cvWork.notify_all();
    return LVBGS_OK;
}

int lvserve_poll(lvserve_handle s, lvserve_result* out, int max, int timeout_ms) {
    if (!s || !out || max <= 0) return 0;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->results.empty() && timeout_ms > 0)
        s->cvDone.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return !s->results.empty(); });
    int n = 0;
    while (n < max && !s->results.empty()) {
        out[n++] = s->results.front();
        s->results.pop_front();
    }
    return n;
}

lvbgs_status lvserve_drain(lvserve_handle s, int timeout_ms) {
    if (!s) return LVBGS_BAD_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    const bool ok = s->cvDone.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] {
        if (s->queued != 0 || s->inflightN != 0 || !s->admitQ.empty()) return false;
        for (auto& kv : s->streams)
            if (kv.second->closing) return false;
        return true;
    });
    return ok ? LVBGS_OK : LVBGS_BUSY;
}

lvbgs_status lvserve_get_stats(lvserve_handle s, lvserve_stats* out) {
    if (!s || !out) return LVBGS_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *out = s->st;
    out->live = (int)s->streams.size();
    out->waiting = (int)s->admitQ.size();
    out->resident = out->spilled = 0;
    for (auto& kv : s->streams) {
        if (kv.second->state == S_RESIDENT) ++out->resident;
        if (kv.second->state == S_SPILLED) ++out->spilled;
    }
    out->device_bytes_in_use = s->used;
    out->mean_tick_streams = s->st.ticks ? s->tickStreamsSum / (double)s->st.ticks : 0.0;
    if (s->inflightN > 0) out->busy_ms += ms_between(s->busySince, Clock::now());
    return LVBGS_OK;
}

double lvserve_latency_quantile(lvserve_handle s, double q) {
    if (!s) return -1.0;
    std::vector<double> v;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        v = s->lat;
    }
    if (v.empty()) return -1.0;
    q = std::min(1.0, std::max(0.0, q));
    const size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)(v.size() - 1) + 0.5));
    std::nth_element(v.begin(), v.begin() + k, v.end());
    return v[k];
}

lvbgs_status lvserve_reset_stats(lvserve_handle s) {
    if (!s) return LVBGS_BAD_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    s->lat.clear();
    s->latPos = 0;
    s->st = lvserve_stats{};
    s->st.peak_device_bytes = s->used;
    s->tickStreamsSum = 0;
    if (s->inflightN > 0) s->busySince = Clock::now();
    return LVBGS_OK;
}

int lvserve_stream_state(lvserve_handle s, int id) {
    if (!s) return S_CLOSED;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->streams.find(id);
    if (it == s->streams.end()) return S_CLOSED;
    return it->second->state == S_INIT ? S_WAITING : it->second->state;
}

const char* lvserve_last_error(lvserve_handle s) {
    if (!s) return "null server";
    std::lock_guard<std::mutex> lk(s->mu);
    static thread_local std::string copy;
    copy = s->err;
    return copy.c_str();
}

int lvserve_plan_room(size_t used, size_t budget, size_t need, const size_t* bytes, const double* idle, int n,
                      double idle_spill_ms, int* out) {
    if (n < 0 || (n > 0 && (!bytes || !idle || !out))) return -1;
    return plan_room(used, budget, need, bytes, idle, n, idle_spill_ms, out);
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// serving workload simulator
// ------------------------------------------------------------------------------------------
namespace {

struct Rng {  // splitmix64: portable, identical on every host
    uint64_t x;
    uint64_t next() {
        uint64_t z = (x += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    double uni() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double expo(double rate) { return -std::log(1.0 - uni()) / rate; }
};

struct SimStream {
    double tArrive = 0, tEnd = 0;
    size_t idx = 0;  // position in the population (frame tags carry it)
    int cls = 0;  // 2 * resolution class + gray
    int W = 0, H = 0, C = 0;
    lvbgs_algo algo = LVBGS_ALGO_SUBSENSE;
    uint64_t seed = 0;
    int id = -1;
    bool rejected = false;
    uint8_t* pool = nullptr;  // pool_frames frames, then one mask
    size_t poolBytes = 0;
    std::atomic<int> ready{0};
    int outstanding = 0;  // frames submitted and not finished (guarded by the server's mutex)
    bool closed = false;
};

struct Slabs {  // pinned buffers per stream class, recycled
    std::mutex mu;
    std::vector<std::vector<uint8_t*>> freeBy{8};
    std::vector<uint8_t*> all;
    uint8_t* get(int cls, size_t bytes) {
        {
            std::lock_guard<std::mutex> lk(mu);
            if (!freeBy[cls].empty()) {
                uint8_t* p = freeBy[cls].back();
                freeBy[cls].pop_back();
                return p;
            }
        }
        void* p = nullptr;
        if (cudaHostAlloc(&p, bytes, cudaHostAllocDefault) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        std::lock_guard<std::mutex> lk(mu);
        all.push_back((uint8_t*)p);
        return (uint8_t*)p;
    }
    void put(int cls, uint8_t* p) {
        std::lock_guard<std::mutex> lk(mu);
        freeBy[cls].push_back(p);
    }
    ~Slabs() {
        for (uint8_t* p : all) cudaFreeHost(p);
    }
};

double quantile(std::vector<double> v, double q) {
    if (v.empty()) return 0.0;
    const size_t k = (size_t)std::min<double>((double)v.size() - 1, std::floor(q * (double)(v.size() - 1) + 0.5));
    std::nth_element(v.begin(), v.begin() + k, v.end());
    return v[k];
}

}  // namespace

extern "C" {

lvbgs_status lvserve_default_sim_config(lvserve_sim_config* o) {
    if (!o) return LVBGS_BAD_ARG;
    *o = lvserve_sim_config{20.0, 3.0, 4.0, 10.0, 60.0, 30.0, {0.3, 0.3, 0.3, 0.1}, 0.25, 0.025, 1, 4, 4, 1};
    return LVBGS_OK;
}

lvbgs_status lvserve_simulate(const lvserve_config* cfg, const lvserve_sim_config* simIn, lvserve_sim_result* out) {
    if (!out) return LVBGS_BAD_ARG;
    std::memset(out, 0, sizeof(*out));
    lvserve_sim_config sim;
    lvserve_default_sim_config(&sim);
    if (simIn) sim = *simIn;
    if (sim.duration_s <= 0 || sim.warmup_s < 0 || sim.arrival_rate < 0 || sim.life_min_s <= 0 ||
        sim.life_max_s < sim.life_min_s || sim.fps <= 0 || sim.pool_frames < 1 || sim.render_threads < 1 ||
        !(sim.pawcs_prob >= 0.0 && sim.pawcs_prob <= 1.0))
        return LVBGS_BAD_ARG;
    static const int kW[4] = {320, 640, 1280, 1920}, kH[4] = {240, 480, 720, 1080};
    const double horizon = sim.warmup_s + sim.duration_s;
    Rng rng{sim.seed * 0x2545F4914F6CDD1Dull + 12345};
    auto draw_stream = [&](double tA) {
        std::unique_ptr<SimStream> z(new SimStream());
        z->tArrive = tA;
        z->tEnd = tA + sim.life_min_s + (sim.life_max_s - sim.life_min_s) * rng.uni();
        const double u = rng.uni();
        double acc = 0;
        int r = 3;
        for (int i = 0; i < 4; ++i) {
            acc += sim.res_prob[i];
            if (u < acc) {
                r = i;
                break;
            }
        }
        const int gray = rng.uni() < sim.gray_prob ? 1 : 0;
        // a share of the streams (of either channel count) run PAWCS
        z->algo = rng.uni() < sim.pawcs_prob ? LVBGS_ALGO_PAWCS : LVBGS_ALGO_SUBSENSE;
        z->cls = 2 * r + gray;
        z->W = kW[r];
        z->H = kH[r];
        z->C = gray ? 1 : 3;
        z->seed = rng.next() >> 8;
        return z;
    };
    // population: arrivals of the past that are still alive at t=0 (the stationary population of
    // the arrival process), then the arrivals of [0, horizon)
    std::vector<std::unique_ptr<SimStream>> ss;
    if (sim.prefill && sim.arrival_rate > 0) {
        for (double t = -sim.life_max_s + rng.expo(sim.arrival_rate); t < 0; t += rng.expo(sim.arrival_rate)) {
            auto z = draw_stream(t);
            if (z->tEnd > 0) ss.push_back(std::move(z));
        }
    }
    const size_t nPrefill = ss.size();
    if (sim.arrival_rate > 0)
        for (double t = rng.expo(sim.arrival_rate); t < horizon; t += rng.expo(sim.arrival_rate))
            ss.push_back(draw_stream(t));
    out->arrivals = ss.size() - nPrefill;
    for (size_t i = 0; i < ss.size(); ++i) ss[i]->idx = i;

    lvserve_handle srv = nullptr;
    lvbgs_status st = lvserve_create(cfg, &srv);
    if (st != LVBGS_OK) return st;
    Slabs slabs;
    const int K = sim.pool_frames;
    // latency records of frames submitted in the measured window (guarded by the server's mutex)
    std::vector<double> lat, admitWait, pawcsLat, subLat;
    uint64_t donePx = 0, doneFrames = 0, pawcsFrames = 0;
    int firstErr = 0;
    Clock::time_point T0;
    std::atomic<bool> clockSet{false};
    const double w0 = sim.warmup_s, w1 = horizon;
    auto in_window = [&](Clock::time_point t) {
        const double s = std::chrono::duration<double>(t - T0).count();
        return s >= w0 && s < w1;
    };
    std::map<int, SimStream*> byId;
    srv->onDone = [&](const SStream& x, const Req& r, Clock::time_point now, int status) {
        if (status != 0 && !firstErr) firstErr = status;
        SimStream* z = ss[(size_t)(r.tag >> 20)].get();
        if (in_window(r.t0)) {
            lat.push_back(ms_between(r.t0, now));
            if (x.algo == LVBGS_ALGO_PAWCS) pawcsLat.push_back(ms_between(r.t0, now));
            else subLat.push_back(ms_between(r.t0, now));
        }
        if (in_window(now)) {
            donePx += x.npx();
            ++doneFrames;
            if (x.algo == LVBGS_ALGO_PAWCS) ++pawcsFrames;
        }
        if (--z->outstanding == 0 && z->closed) slabs.put(z->cls, z->pool);
    };
    srv->onAdmit = [&](const SStream& x, Clock::time_point now) {
        if (clockSet && in_window(now)) admitWait.push_back(ms_between(x.tOpen, now));
    };
    // renderers: pool frames of each stream, in arrival order, a few seconds ahead of the clock
    std::atomic<size_t> nextRender{0};
    std::atomic<bool> abortRender{false};
    std::atomic<int> renderErr{0};
    auto renderer = [&]() {
        for (;;) {
            const size_t i = nextRender.fetch_add(1);
            if (i >= ss.size() || abortRender) return;
            SimStream* z = ss[i].get();
            while (i >= nPrefill && !abortRender) {
                if (clockSet) {
                    const double now = std::chrono::duration<double>(Clock::now() - T0).count();
                    if (z->tArrive - now < 3.0) break;
                }
                std::this_thread::sleep_for(std::chrono::milliseconds(20));
            }
            if (abortRender) return;
            const size_t fb = (size_t)z->W * z->H * z->C;
            z->poolBytes = fb * K + (size_t)z->W * z->H;
            z->pool = slabs.get(z->cls, z->poolBytes);
            lvsynth_config sc;
            lvsynth_handle sh = nullptr;
            if (!z->pool || lvsynth_preset(4, z->cls, z->seed, &sc) != LVBGS_OK || lvsynth_create(&sc, &sh) != LVBGS_OK) {
                renderErr = LVBGS_OOM;
                z->ready = -1;
                continue;
            }
            for (int k = 0; k < K; ++k) lvsynth_render(sh, k, z->pool + fb * k, nullptr);
            lvsynth_destroy(sh);
            z->ready = 1;
        }
    };
    std::vector<std::thread> rth;
    for (int i = 0; i < sim.render_threads; ++i) rth.emplace_back(renderer);
    // the prefill population is rendered before the clock starts
    for (size_t i = 0; i < nPrefill; ++i)
        while (ss[i]->ready == 0) std::this_thread::sleep_for(std::chrono::milliseconds(2));

    // event loop: (time, kind, stream, frame index); kinds 0 open, 1 frame, 2 close, 3 sample
    struct Ev {
        double t;
        int kind;
        SimStream* z;
        int k;
        bool operator>(const Ev& o) const { return t > o.t; }
    };
    std::priority_queue<Ev, std::vector<Ev>, std::greater<Ev>> pq;
    for (auto& zp : ss) {
        SimStream* z = zp.get();
        pq.push({std::max(0.0, z->tArrive), 0, z, 0});
    }
    for (double t = w0; t < w1; t += 0.1) pq.push({t, 3, nullptr, 0});
    double liveSum = 0, resSum = 0;
    int samples = 0, peakLive = 0;
    uint64_t offeredPx = 0, dropped = 0, late = 0, rejected = 0;
    lvserve_stats s0{}, s1{};
    bool haveS0 = false;
    const double dt = 1.0 / sim.fps;
    T0 = Clock::now() + std::chrono::milliseconds(50);
    clockSet = true;
    while (!pq.empty()) {
        const Ev e = pq.top();
        if (e.t >= w1) break;
        pq.pop();
        const Clock::time_point when = T0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(e.t));
        std::this_thread::sleep_until(when);
        const Clock::time_point now = Clock::now();
        if (!haveS0 && e.t >= w0) {
            lvserve_get_stats(srv, &s0);
            haveS0 = true;
        }
        SimStream* z = e.z;
        if (e.kind == 3) {
            lvserve_stats sn;
            lvserve_get_stats(srv, &sn);
            liveSum += sn.live;
            resSum += sn.resident;
            peakLive = std::max(peakLive, sn.live);
            ++samples;
            continue;
        }
        if (e.kind == 0) {
            while (z->ready == 0) std::this_thread::sleep_for(std::chrono::microseconds(200));
            if (z->ready < 0) continue;
            int id = -1;
            lvbgs_params prm;
            lvbgs_default_params(z->algo, &prm);
            prm.seed = z->seed;
            const lvbgs_status r = lvserve_open(srv, z->algo, &prm, z->pool, z->W, z->H, z->C, 0, nullptr, &id);
            if (r != LVBGS_OK) {
                z->rejected = true;
                ++rejected;
                std::lock_guard<std::mutex> lk(srv->mu);
                z->closed = true;
                if (z->outstanding == 0) slabs.put(z->cls, z->pool);
                continue;
            }
            z->id = id;
            // first frame at the next frame time after the arrival (or after t=0 for the prefill)
            const double first = z->tArrive + dt * std::floor((std::max(0.0, z->tArrive) - z->tArrive) / dt + 1.0);
            pq.push({first, 1, z, (int)std::floor((first - z->tArrive) / dt + 0.5)});
            pq.push({z->tEnd, 2, z, 0});
            continue;
        }
        if (e.kind == 2) {
            lvserve_close(srv, z->id);
            std::lock_guard<std::mutex> lk(srv->mu);
            z->closed = true;
            if (z->outstanding == 0) slabs.put(z->cls, z->pool);
            continue;
        }
        // a frame: the pool is replayed forth and back (0,1,..,K-1,K-2,..,1,0,1,...)
        if (e.t >= z->tEnd) continue;
        if (ms_between(when, now) > 5.0) ++late;
        const int period = K > 1 ? 2 * (K - 1) : 1;
        int f = e.k % period;
        if (f >= K) f = period - f;
        const size_t fb = (size_t)z->W * z->H * z->C;
        {
            std::lock_guard<std::mutex> lk(srv->mu);
            ++z->outstanding;
        }
        const uint64_t tag = ((uint64_t)z->idx << 20) | (uint64_t)(e.k & 0xfffff);
        const lvbgs_status r = lvserve_submit(srv, z->id, z->pool + fb * f, 0, z->pool + fb * K, 0.0, tag);
        if (r != LVBGS_OK) {
            ++dropped;
            std::lock_guard<std::mutex> lk(srv->mu);
            --z->outstanding;
        } else if (e.t >= w0) {
            offeredPx += (uint64_t)z->W * z->H;
        }
        pq.push({e.t + dt, 1, z, e.k + 1});
    }
    lvserve_get_stats(srv, &s1);
    abortRender = true;
    for (auto& t : rth) t.join();
    // close everything and let the queued frames finish
    for (auto& zp : ss)
        if (zp->id >= 0 && !zp->closed) {
            lvserve_close(srv, zp->id);
            std::lock_guard<std::mutex> lk(srv->mu);
            zp->closed = true;
            if (zp->outstanding == 0 && zp->pool) slabs.put(zp->cls, zp->pool);
        }
    lvserve_drain(srv, 120000);
    {
        std::lock_guard<std::mutex> lk(srv->mu);
        out->frames = doneFrames;
        out->window_s = sim.duration_s;
        out->mpix_per_s = (double)donePx / 1e6 / sim.duration_s;
        out->frames_per_s = (double)doneFrames / sim.duration_s;
        out->p50_ms = quantile(lat, 0.50);
        out->p90_ms = quantile(lat, 0.90);
        out->p99_ms = quantile(lat, 0.99);
        out->max_ms = lat.empty() ? 0.0 : *std::max_element(lat.begin(), lat.end());
        out->admit_wait_p50_ms = quantile(admitWait, 0.50);
        out->admit_wait_p99_ms = quantile(admitWait, 0.99);
        out->pawcs_p50_ms = quantile(pawcsLat, 0.50);
        out->pawcs_p99_ms = quantile(pawcsLat, 0.99);
        out->pawcs_frames = pawcsFrames;
        out->subsense_p50_ms = quantile(subLat, 0.50);
        out->subsense_p99_ms = quantile(subLat, 0.99);
        out->status = firstErr;
    }
    out->offered_mpix_per_s = (double)offeredPx / 1e6 / sim.duration_s;
    out->mean_live = samples ? liveSum / samples : 0.0;
    out->mean_resident = samples ? resSum / samples : 0.0;
    out->peak_live = peakLive;
    out->ticks = s1.ticks - s0.ticks;
    out->mean_tick_streams = out->ticks ? (s1.mean_tick_streams * s1.ticks - s0.mean_tick_streams * s0.ticks) / out->ticks : 0.0;
    out->gpu_busy_frac = (s1.busy_ms - s0.busy_ms) / (sim.duration_s * 1e3);
    out->admitted = s1.admitted;
    out->rejected = rejected;
    out->dropped = dropped;
    out->spills = s1.spills;
    out->restores = s1.restores;
    out->late_frames = late;
    out->peak_device_bytes = s1.peak_device_bytes;
    if (!out->status && renderErr) out->status = renderErr;
    srv->onDone = nullptr;
    srv->onAdmit = nullptr;
    lvserve_destroy(srv);
    return LVBGS_OK;
}

}  // extern "C"
