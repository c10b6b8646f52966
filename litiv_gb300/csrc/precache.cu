// Frame precacher: lv::DataPrecacher (modules/datasets/include/litiv/datasets/utils.hpp:456-478,
// modules/datasets/src/utils.cpp:302-470) for a GPU consumer.
//
// The reference's precacher runs the packet loader on a thread ahead of the requests and keeps the
// loaded packets in a host ring buffer; getPacket(idx) hands out the requested packet, sequential
// requests being served from the ring, others loaded on demand, and an empty packet ending the stream.
// Here the ring has slots of pinned host memory, each with a device twin: the worker thread fills the
// next free slot with the loader, copies it to the device on a dedicated copy stream and records a
// "ready" event, so the upload of packet i+1.. overlaps the caller's work on packet i. get() makes the
// caller's stream wait on the packet's ready event (no host wait when it is already loaded) and hands
// out the device and host pointers. The previously handed packet is released at the next get(): a
// "release" event recorded on the caller's stream there orders the next upload into that device slot
// after everything the caller enqueued before (the copy stream waits on it; the host is never blocked).
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/lvbgs.h"
#include "lvbgs_internal.h"

namespace {

constexpr int kMinSlots = 2, kMaxSlots = 64;
constexpr int kRequestTimeoutMs = 100;  // a request re-checks the worker's state this often while it waits

struct Slot {
    uint8_t* host = nullptr;
    uint8_t* dev = nullptr;
    size_t idx = SIZE_MAX, size = 0;
    const uint8_t* src = nullptr;  // the host copy of the packet (the slot's buffer or the caller's memory)
    enum State { FREE, LOADING, READY, HANDED } state = FREE;
    cudaEvent_t ready = nullptr, release = nullptr;
    bool released = false;  // `release` holds the last consumer use of the device buffer
};

}  // namespace

struct lvbgs_precacher_ctx {
    lvbgs_packet_loader loader = nullptr;
    void* user = nullptr;
    // packets already in the caller's host memory (lvbgs_precacher_create_host): uploaded from there,
    // with no loader and no host slots
    const uint8_t* direct = nullptr;
    size_t directCount = 0;
    size_t cap = 0;
    int device = 0;
    std::vector<Slot> slots;
    cudaStream_t copy = nullptr;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cvWork, cvReady;
    bool active = false, stopping = false;
    size_t nextIdx = 0;          // next packet the worker loads
    size_t endIdx = SIZE_MAX;    // first index whose load came back empty
    size_t lastReq = SIZE_MAX;   // last requested index (getLastReqIdx)
    int handed = -1;             // slot of the last handed packet
    std::string workerError;     // set by the worker: the loader failed
    std::string err;

    void run();
    int find(size_t idx) const {
        for (size_t i = 0; i < slots.size(); ++i)
            if ((slots[i].state == Slot::READY || slots[i].state == Slot::LOADING || slots[i].state == Slot::HANDED) &&
                slots[i].idx == idx)
                return (int)i;
        return -1;
    }
};

namespace {

lvbgs_status pfail(lvbgs_precacher p, lvbgs_status st, const std::string& msg) {
    if (p) p->err = msg;
    return lvbgs::report_error(st, msg.c_str());
}

void free_slots(lvbgs_precacher p) {
    for (Slot& s : p->slots) {
        if (s.host) cudaFreeHost(s.host);
        if (s.dev) cudaFree(s.dev);
        if (s.ready) cudaEventDestroy(s.ready);
        if (s.release) cudaEventDestroy(s.release);
    }
    p->slots.clear();
}

lvbgs_status alloc_slots(lvbgs_precacher p, int n) {
    p->slots.resize((size_t)n);
    for (Slot& s : p->slots) {
        if ((!p->direct && cudaHostAlloc((void**)&s.host, p->cap, cudaHostAllocDefault) != cudaSuccess) ||
            cudaMalloc(&s.dev, p->cap) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.ready, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&s.release, cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            free_slots(p);
            return pfail(p, LVBGS_OOM, "precacher slot allocation failed");
        }
    }
    return LVBGS_OK;
}

// stops the worker (joins it) and clears the ring; the caller holds no lock
void stop_worker(lvbgs_precacher p) {
    {
        std::lock_guard<std::mutex> lk(p->mu);
        if (!p->active) return;
        p->stopping = true;
    }
    p->cvWork.notify_all();
    if (p->worker.joinable()) p->worker.join();
    cudaStreamSynchronize(p->copy);
    std::lock_guard<std::mutex> lk(p->mu);
    p->active = false;
    p->stopping = false;
}

}  // namespace

// the precaching thread (DataPrecacher::entry, utils.cpp:388-470): loads the packets after the last
// request into free slots, in order, until the stream ends or the ring is full
void lvbgs_precacher_ctx::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (!stopping) {
        int free = -1;
        if (nextIdx < endIdx)
            for (size_t i = 0; i < slots.size(); ++i)
                if (slots[i].state == Slot::FREE) {
                    free = (int)i;
                    break;
                }
        if (free < 0) {
            cvWork.wait_for(lk, std::chrono::milliseconds(20));
            continue;
        }
        Slot& s = slots[(size_t)free];
        const size_t idx = nextIdx++;
        s.state = Slot::LOADING;
        s.idx = idx;
        lk.unlock();
        size_t size;
        const uint8_t* src;
        if (direct) {
            size = idx < directCount ? cap : 0;
            src = direct + idx * cap;
        } else {
            // the host buffer's previous upload has finished long before a slot is free again; wait for it anyway
            cudaEventSynchronize(s.ready);
            size = loader(user, idx, s.host, cap);
            src = s.host;
        }
        cudaError_t e = cudaSuccess;
        if (size != 0 && size <= cap) {
            if (s.released) e = cudaStreamWaitEvent(copy, s.release, 0);
            if (e == cudaSuccess) e = cudaMemcpyAsync(s.dev, src, size, cudaMemcpyHostToDevice, copy);
            if (e == cudaSuccess) e = cudaEventRecord(s.ready, copy);
        }
        lk.lock();
        if (size == 0) {
            // an empty packet ends the stream (utils.hpp:458)
            endIdx = std::min(endIdx, idx);
            s.state = Slot::FREE;
            s.idx = SIZE_MAX;
        } else if (size > cap || e != cudaSuccess) {
            workerError = size > cap ? "the loader returned a packet larger than the precacher's packet capacity"
                                     : std::string("packet upload failed: ") + cudaGetErrorString(e);
            s.state = Slot::FREE;
            s.idx = SIZE_MAX;
            cvReady.notify_all();
            break;
        } else {
            s.size = size;
            s.src = src;
            s.state = Slot::READY;
        }
        cvReady.notify_all();
    }
}

extern "C" {

size_t lvbgs_precache_copy_loader(void* user, size_t idx, uint8_t* dst, size_t cap) {
    const lvbgs_host_packets* a = (const lvbgs_host_packets*)user;
    if (!a || idx >= a->count) return 0;
    const size_t n = std::min(a->packet_bytes, cap);
    std::memcpy(dst, a->base + idx * a->packet_bytes, n);
    return a->packet_bytes;
}

lvbgs_status lvbgs_precacher_create(lvbgs_packet_loader loader, void* user, size_t max_packet_bytes, int device_id,
                                    lvbgs_precacher* out) {
    if (!out) return pfail(nullptr, LVBGS_BAD_ARG, "null output");
    *out = nullptr;
    // DataPrecacher(lDataLoaderCallback) (utils.cpp:302-308): the callback must be valid
    if (!loader) return pfail(nullptr, LVBGS_BAD_ARG, "invalid data precacher callback");
    if (max_packet_bytes == 0) return pfail(nullptr, LVBGS_BAD_ARG, "packet capacity must be positive");
    if (cudaSetDevice(device_id) != cudaSuccess) {
        cudaGetLastError();
        return pfail(nullptr, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    }
    lvbgs_precacher p = new lvbgs_precacher_ctx();
    p->loader = loader;
    p->user = user;
    p->cap = max_packet_bytes;
    p->device = device_id;
    if (cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return pfail(nullptr, LVBGS_DEVICE_ERROR, "stream creation failed");
    }
    // one slot for requests made while precaching is off
    lvbgs_status s = alloc_slots(p, 1);
    if (s != LVBGS_OK) {
        cudaStreamDestroy(p->copy);
        delete p;
        return s;
    }
    *out = p;
    return LVBGS_OK;
}

lvbgs_status lvbgs_precacher_create_host(const uint8_t* packets, size_t packet_bytes, size_t count, int device_id,
                                         lvbgs_precacher* out) {
    if (!out) return pfail(nullptr, LVBGS_BAD_ARG, "null output");
    *out = nullptr;
    if (!packets || packet_bytes == 0) return pfail(nullptr, LVBGS_BAD_ARG, "packets and a positive packet size are required");
    if (cudaSetDevice(device_id) != cudaSuccess) {
        cudaGetLastError();
        return pfail(nullptr, LVBGS_DEVICE_ERROR, "cannot select the CUDA device");
    }
    lvbgs_precacher p = new lvbgs_precacher_ctx();
    p->direct = packets;
    p->directCount = count;
    p->cap = packet_bytes;
    p->device = device_id;
    if (cudaStreamCreateWithFlags(&p->copy, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        delete p;
        return pfail(nullptr, LVBGS_DEVICE_ERROR, "stream creation failed");
    }
    lvbgs_status s = alloc_slots(p, 1);
    if (s != LVBGS_OK) {
        cudaStreamDestroy(p->copy);
        delete p;
        return s;
    }
    *out = p;
    return LVBGS_OK;
}

lvbgs_status lvbgs_precacher_destroy(lvbgs_precacher p) {
    if (!p) return LVBGS_OK;
    cudaSetDevice(p->device);
    stop_worker(p);
    cudaStreamSynchronize(p->copy);
    cudaDeviceSynchronize();  // packets handed out may still be read by the caller's streams
    free_slots(p);
    cudaStreamDestroy(p->copy);
    delete p;
    return LVBGS_OK;
}

// startAsyncPrecaching(nSuggestedBufferSize) (utils.cpp:358-374): a ring of buffer_bytes / packet
// capacity slots (2..64), empty, filled from packet 0 on. A ring of the same size as the last one is
// reused (the allocation of pinned slots is slow)
lvbgs_status lvbgs_precacher_start(lvbgs_precacher p, size_t buffer_bytes) {
    if (!p) return pfail(nullptr, LVBGS_BAD_ARG, "null precacher");
    cudaSetDevice(p->device);
    stop_worker(p);
    if (buffer_bytes == 0) return LVBGS_OK;
    const size_t want = buffer_bytes / p->cap;
    const int n = (int)std::max<size_t>(kMinSlots, std::min<size_t>(kMaxSlots, want));
    // packets handed out before may still be read by the caller's streams
    cudaDeviceSynchronize();
    if ((int)p->slots.size() != n) {
        free_slots(p);
        lvbgs_status s = alloc_slots(p, n);
        if (s != LVBGS_OK) {
            alloc_slots(p, 1);
            return s;
        }
    }
    std::lock_guard<std::mutex> lk(p->mu);
    for (Slot& sl : p->slots) {
        sl.state = Slot::FREE;
        sl.idx = SIZE_MAX;
        sl.released = false;
    }
    p->handed = -1;
    p->lastReq = SIZE_MAX;
    p->nextIdx = 0;
    p->endIdx = SIZE_MAX;
    p->workerError.clear();
    p->active = true;
    p->stopping = false;
    p->worker = std::thread([p] { p->run(); });
    return LVBGS_OK;
}

// stopAsyncPrecaching() (utils.cpp:376-386): joins the worker and empties the ring (its slots stay
// allocated for the next start); reports a loader error the worker met (the reference rethrows it)
lvbgs_status lvbgs_precacher_stop(lvbgs_precacher p) {
    if (!p) return pfail(nullptr, LVBGS_BAD_ARG, "null precacher");
    cudaSetDevice(p->device);
    stop_worker(p);
    cudaDeviceSynchronize();
    std::lock_guard<std::mutex> lk(p->mu);
    for (Slot& sl : p->slots) {
        sl.state = Slot::FREE;
        sl.idx = SIZE_MAX;
        sl.released = false;
    }
    p->handed = -1;
    p->lastReq = SIZE_MAX;
    const std::string werr = p->workerError;
    p->workerError.clear();
    // the reference rethrows a worker exception here (utils.cpp:384-385)
    if (!werr.empty()) return pfail(p, LVBGS_BAD_ARG, werr);
    return LVBGS_OK;
}

int lvbgs_precacher_is_active(lvbgs_precacher p) {
    if (!p) return 0;
    std::lock_guard<std::mutex> lk(p->mu);
    return p->active ? 1 : 0;
}

size_t lvbgs_precacher_last_index(lvbgs_precacher p) {
    if (!p) return SIZE_MAX;
    std::lock_guard<std::mutex> lk(p->mu);
    return p->lastReq;
}

// getPacket(idx) (utils.cpp:314-356)
lvbgs_status lvbgs_precacher_get(lvbgs_precacher p, size_t idx, void* cuda_stream, const uint8_t** device_packet,
                                 const uint8_t** host_packet, size_t* size) {
    if (!p || !size) return pfail(p, LVBGS_BAD_ARG, "null argument");
    cudaSetDevice(p->device);
    cudaStream_t st = (cudaStream_t)cuda_stream;
    std::unique_lock<std::mutex> lk(p->mu);
    auto hand = [&](int i) -> lvbgs_status {
        Slot& s = p->slots[(size_t)i];
        if (cudaStreamWaitEvent(st, s.ready, 0) != cudaSuccess) {
            cudaGetLastError();
            return pfail(p, LVBGS_DEVICE_ERROR, "cannot order the caller's stream after the packet upload");
        }
        if (device_packet) *device_packet = s.dev;
        if (host_packet) *host_packet = s.src;
        *size = s.size;
        p->lastReq = idx;
        return LVBGS_OK;
    };
    // the same packet again (utils.cpp:316-319)
    if (p->handed >= 0 && idx == p->lastReq) return hand(p->handed);
    // release the previous packet: the caller's work enqueued so far on its stream may still read it
    if (p->handed >= 0) {
        Slot& s = p->slots[(size_t)p->handed];
        cudaEventRecord(s.release, st);
        s.released = true;
        s.state = Slot::FREE;
        s.idx = SIZE_MAX;
        p->handed = -1;
    }
    if (!p->active) {
        // no precaching (utils.cpp:320-325): load into the single slot, synchronously
        Slot& s = p->slots[0];
        lk.unlock();
        size_t n;
        if (p->direct) {
            n = idx < p->directCount ? p->cap : 0;
            s.src = p->direct + idx * p->cap;
        } else {
            cudaEventSynchronize(s.ready);  // the host buffer's last upload
            n = p->loader(p->user, idx, s.host, p->cap);
            s.src = s.host;
        }
        lk.lock();
        if (n > p->cap) return pfail(p, LVBGS_BAD_ARG, "the loader returned a packet larger than the precacher's packet capacity");
        s.size = n;
        s.idx = idx;
        if (n == 0) {
            if (device_packet) *device_packet = nullptr;
            if (host_packet) *host_packet = nullptr;
            *size = 0;
            p->lastReq = idx;
            return LVBGS_OK;
        }
        if ((s.released && cudaStreamWaitEvent(p->copy, s.release, 0) != cudaSuccess) ||
            cudaMemcpyAsync(s.dev, s.src, n, cudaMemcpyHostToDevice, p->copy) != cudaSuccess ||
            cudaEventRecord(s.ready, p->copy) != cudaSuccess) {
            cudaGetLastError();
            return pfail(p, LVBGS_DEVICE_ERROR, "packet upload failed");
        }
        s.state = Slot::HANDED;
        p->handed = 0;
        return hand(0);
    }
    // a request outside the precached window restarts the worker's sequence there
    if (p->find(idx) < 0 && idx != p->nextIdx) {
        for (Slot& s : p->slots)
            if (s.state == Slot::READY) {
                s.state = Slot::FREE;
                s.idx = SIZE_MAX;
            }
        p->nextIdx = idx;
        if (idx < p->endIdx) p->endIdx = SIZE_MAX;
        p->cvWork.notify_all();
    }
    for (;;) {
        if (idx >= p->endIdx) {
            // past the end of the stream: an empty packet
            if (device_packet) *device_packet = nullptr;
            if (host_packet) *host_packet = nullptr;
            *size = 0;
            p->lastReq = idx;
            return LVBGS_OK;
        }
        const int i = p->find(idx);
        if (i >= 0 && p->slots[(size_t)i].state == Slot::READY) {
            p->slots[(size_t)i].state = Slot::HANDED;
            p->handed = i;
            // packets before this one (left over from a restarted sequence) are not requested again
            for (Slot& o : p->slots)
                if (o.state == Slot::READY && o.idx < idx) {
                    o.state = Slot::FREE;
                    o.idx = SIZE_MAX;
                }
            p->cvWork.notify_all();
            return hand(i);
        }
        // a failed worker has stopped: the packets it loaded before the failing one are still served
        if (!p->workerError.empty()) return pfail(p, LVBGS_BAD_ARG, p->workerError);
        if (i < 0 && idx >= p->nextIdx) {
            // not yet scheduled: make it the next load (the worker only moves forward)
            p->nextIdx = idx;
            p->cvWork.notify_all();
        }
        p->cvReady.wait_for(lk, std::chrono::milliseconds(kRequestTimeoutMs));
    }
}

}  // extern "C"
