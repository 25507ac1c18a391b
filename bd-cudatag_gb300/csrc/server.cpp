// Continuous-batching detection server (no counterpart in the reference).
//
// Frames from several cameras arrive at any time.  A scheduler thread keeps
// a fixed set of batch plans (one slot per camera, created up front inside a
// device-memory budget -- that budget is the admission limit) and, whenever
// a plan is free, launches it with the oldest waiting frame of every camera
// that has one; cameras without a waiting frame leave their slot out of that
// launch.  Frames that arrive while batches run join the next launch, and
// up to `plans` batches run on the GPU at once on separate streams.  Each
// frame's result is the result a bd_detector of its camera's size returns
// for it (the kernels of a slot do not depend on the other slots).

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "bdcudatag/bdcudatag.h"
#include "bdcudatag/bdcudatag_gb300.h"
#include "engine.h"
#include "pipeline.cuh"

namespace bdgb {
void set_last_error(const char* message);  // capi.cpp
}

namespace {

using Clock = std::chrono::steady_clock;

struct Request {
    int camera = 0;
    const uint8_t* frame = nullptr;   // caller memory (page-locked) or `owned`
    int stride = 0;
    uint8_t* owned = nullptr;         // pinned copy of a pageable frame
    Clock::time_point arrival;
    Clock::time_point done_at;
    bool done = false;
    int32_t found[2] = {-1, -1};
    std::vector<bd_detection> dets;   // 2 * max_detections
};

}  // namespace

struct bd_server {
    std::vector<bd_camera> cameras;
    std::vector<bdgb::Plan*> plans;
    std::vector<std::vector<int64_t>> slot_ticket;   // per plan, per camera: ticket or -1
    std::vector<bool> plan_busy;
    std::vector<std::deque<int64_t>> pending;        // per camera, FIFO
    std::vector<std::vector<uint8_t*>> free_buffers; // per camera pinned request buffers
    std::vector<int> outstanding;                    // per camera: requests not yet collected
    std::unordered_map<int64_t, Request> requests;
    int queue_depth = 0;
    int max_detections = 0;
    int device = 0;
    int64_t next_ticket = 0;
    std::mutex mutex;
    std::condition_variable work_cv;
    std::condition_variable done_cv;
    std::thread scheduler;
    bool stop = false;
    std::string fatal;
    // statistics
    uint64_t submitted = 0, completed = 0, rejected = 0, batches = 0, batched_frames = 0;
    int peak_inflight = 0;
    int64_t device_bytes = 0;

    void run();
    void finish_plan(int p);
};

void bd_server::finish_plan(int p) {
    bdgb::Plan& plan = *plans[p];
    std::string error;
    const bool ok = plan.wait(&error) == 0;
    if (!ok) fatal = error;  // every collect reports it; no result is read
    const auto now = Clock::now();
    for (size_t c = 0; c < cameras.size(); ++c) {
        const int64_t t = slot_ticket[p][c];
        if (t < 0) continue;
        slot_ticket[p][c] = -1;
        auto it = requests.find(t);
        if (it == requests.end()) continue;
        Request& r = it->second;
        for (int f = 0; ok && f < 2; ++f) {
            if (!((cameras[c].families >> f) & 1u)) continue;
            const int n = std::max(0, std::min(plan.found(static_cast<int>(c), f), max_detections));
            r.found[f] = n;
            std::memcpy(r.dets.data() + static_cast<size_t>(f) * max_detections,
                        plan.detections(static_cast<int>(c), f), sizeof(bd_detection) * n);
        }
        r.done = true;
        r.done_at = now;
        if (r.owned) {
            free_buffers[c].push_back(r.owned);
            r.owned = nullptr;
        }
        ++completed;
    }
    plan_busy[p] = false;
}

void bd_server::run() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(mutex);
    std::vector<const uint8_t*> frames(cameras.size());
    std::vector<int32_t> strides(cameras.size());
    while (!stop) {
        bool progress = false;
        int inflight = 0;
        for (size_t p = 0; p < plans.size(); ++p) {
            if (!plan_busy[p]) continue;
            std::string error;
            const int q = plans[p]->query(&error);
            if (q != 0) {
                if (q < 0) fatal = error;
                finish_plan(static_cast<int>(p));
                progress = true;
            } else {
                ++inflight;
            }
        }
        for (size_t p = 0; p < plans.size(); ++p) {
            if (plan_busy[p]) continue;
            bool any = false;
            for (size_t c = 0; c < cameras.size(); ++c) {
                frames[c] = nullptr;
                strides[c] = cameras[c].width;
                slot_ticket[p][c] = -1;
                if (pending[c].empty()) continue;
                const int64_t t = pending[c].front();
                pending[c].pop_front();
                const Request& r = requests[t];
                frames[c] = r.frame;
                strides[c] = r.stride;
                slot_ticket[p][c] = t;
                any = true;
                ++batched_frames;
            }
            if (!any) break;
            std::string error;
            if (plans[p]->submit_slots(frames.data(), strides.data(), &error) != 0) {
                fatal = error;
                for (size_t c = 0; c < cameras.size(); ++c) {
                    if (slot_ticket[p][c] >= 0) requests[slot_ticket[p][c]].done = true;
                    slot_ticket[p][c] = -1;
                }
                continue;
            }
            plan_busy[p] = true;
            ++batches;
            ++inflight;
            progress = true;
        }
        peak_inflight = std::max(peak_inflight, inflight);
        if (progress) done_cv.notify_all();
        if (inflight == 0) {
            work_cv.wait_for(lock, std::chrono::milliseconds(2));
        } else if (!progress) {
            lock.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(10));
            lock.lock();
        }
    }
}

namespace {

void release_server(bd_server* s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lock(s->mutex);
        s->stop = true;
    }
    s->work_cv.notify_all();
    if (s->scheduler.joinable()) s->scheduler.join();
    for (bdgb::Plan* p : s->plans) delete p;
    for (auto& list : s->free_buffers) {
        for (uint8_t* b : list) cudaFreeHost(b);
    }
    for (auto& kv : s->requests) {
        if (kv.second.owned) cudaFreeHost(kv.second.owned);
    }
    delete s;
}

int32_t collect(bd_server* s, int64_t ticket, bool block, bd_detection* out, int32_t* found,
                double* latency_ms) {
    if (!s) {
        bdgb::set_last_error("null server");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    std::unique_lock<std::mutex> lock(s->mutex);
    auto it = s->requests.find(ticket);
    if (it == s->requests.end()) {
        bdgb::set_last_error("unknown or already collected ticket");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    while (!it->second.done) {
        if (!block) return 0;
        s->done_cv.wait(lock);
        it = s->requests.find(ticket);
    }
    if (!s->fatal.empty()) {
        bdgb::set_last_error(s->fatal.c_str());
        return BD_ERROR_CUDA;
    }
    Request& r = it->second;
    if (found) {
        found[0] = r.found[0];
        found[1] = r.found[1];
    }
    if (out) {
        std::memcpy(out, r.dets.data(), sizeof(bd_detection) * r.dets.size());
    }
    if (latency_ms) {
        *latency_ms = std::chrono::duration<double, std::milli>(r.done_at - r.arrival).count();
    }
    s->outstanding[r.camera] -= 1;
    s->requests.erase(it);
    return 1;
}

}  // namespace

extern "C" {

bd_server* bd_server_create(const bd_camera* cameras, int32_t count, const bd_config* config,
                            int64_t device_budget_bytes, int32_t max_batches, int32_t queue_depth,
                            int32_t* status_out) {
    if (status_out) *status_out = BD_OK;
    if (!cameras || count < 1 || count > BD_BATCH_MAX_CAMERAS || max_batches < 1 || queue_depth < 1) {
        bdgb::set_last_error("bd_server_create: bad camera list, batch count or queue depth");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    if (config && config->struct_size != 0 && config->struct_size < sizeof(bd_config)) {
        bdgb::set_last_error("bd_config.struct_size is too small for this library version");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    std::vector<bdgb::PlanFrame> frames(count);
    for (int i = 0; i < count; ++i) {
        if (cameras[i].width < 16 || cameras[i].width > BD_MAX_WIDTH || cameras[i].height < 16 ||
            cameras[i].height > BD_MAX_HEIGHT || (cameras[i].families & 3u) == 0 ||
            (cameras[i].families & ~3u) != 0) {
            bdgb::set_last_error("bd_server_create: camera size or family mask out of range");
            if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
            return nullptr;
        }
        frames[i].width = cameras[i].width;
        frames[i].height = cameras[i].height;
        frames[i].families = cameras[i].families;
    }
    bd_server* s = new (std::nothrow) bd_server();
    if (!s) {
        if (status_out) *status_out = BD_ERROR_OUT_OF_MEMORY;
        return nullptr;
    }
    s->cameras.assign(cameras, cameras + count);
    cudaGetDevice(&s->device);
    const bdgb::PlanConfig pc = bdgb::resolve_config(config);
    s->max_detections = pc.max_detections;
    s->queue_depth = queue_depth;
    // Admission by memory: as many batch plans as the budget holds.
    std::string error;
    for (int p = 0; p < max_batches; ++p) {
        if (p > 0 && s->device_bytes + s->device_bytes / p > device_budget_bytes) break;
        bdgb::Plan* plan = bdgb::Plan::create(frames, pc, &error);
        if (!plan) break;
        if (p == 0 && static_cast<int64_t>(plan->device_bytes()) > device_budget_bytes) {
            delete plan;
            error = "device budget is smaller than one batch";
            break;
        }
        s->device_bytes += static_cast<int64_t>(plan->device_bytes());
        s->plans.push_back(plan);
    }
    if (s->plans.empty()) {
        bdgb::set_last_error(("bd_server_create: " + error).c_str());
        if (status_out) *status_out = BD_ERROR_OUT_OF_MEMORY;
        release_server(s);
        return nullptr;
    }
    const size_t np = s->plans.size();
    s->slot_ticket.assign(np, std::vector<int64_t>(count, -1));
    s->plan_busy.assign(np, false);
    s->pending.resize(count);
    s->free_buffers.resize(count);
    s->outstanding.assign(count, 0);
    for (int c = 0; c < count; ++c) {
        for (int k = 0; k < queue_depth; ++k) {
            uint8_t* buf = nullptr;
            if (cudaHostAlloc(reinterpret_cast<void**>(&buf),
                              static_cast<size_t>(cameras[c].width) * cameras[c].height,
                              cudaHostAllocPortable) != cudaSuccess) {
                cudaGetLastError();
                bdgb::set_last_error("bd_server_create: cudaHostAlloc failed");
                if (status_out) *status_out = BD_ERROR_OUT_OF_MEMORY;
                release_server(s);
                return nullptr;
            }
            s->free_buffers[c].push_back(buf);
        }
    }
    s->scheduler = std::thread([s] { s->run(); });
    return s;
}

void bd_server_destroy(bd_server* server) { release_server(server); }

int64_t bd_server_submit(bd_server* s, int32_t camera, const uint8_t* gray, int32_t stride) {
    if (!s || camera < 0 || camera >= static_cast<int32_t>(s->cameras.size()) || !gray) {
        bdgb::set_last_error("bd_server_submit: bad server, camera or frame");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const bd_camera& cam = s->cameras[camera];
    if (stride < cam.width) {
        bdgb::set_last_error("stride is smaller than the image width");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const auto arrival = Clock::now();
    cudaPointerAttributes attr;
    const bool pinned = cudaPointerGetAttributes(&attr, gray) == cudaSuccess &&
                        attr.type == cudaMemoryTypeHost;
    cudaGetLastError();
    std::unique_lock<std::mutex> lock(s->mutex);
    if (s->outstanding[camera] >= s->queue_depth || (!pinned && s->free_buffers[camera].empty())) {
        ++s->rejected;
        bdgb::set_last_error("bd_server_submit: camera queue is full");
        return BD_ERROR_OUT_OF_MEMORY;
    }
    s->outstanding[camera] += 1;  // reserved before the lock is released for a copy
    Request r;
    r.camera = camera;
    r.arrival = arrival;
    r.dets.resize(2 * static_cast<size_t>(s->max_detections));
    if (pinned) {
        r.frame = gray;
        r.stride = stride;
    } else {
        r.owned = s->free_buffers[camera].back();
        s->free_buffers[camera].pop_back();
        lock.unlock();
        for (int y = 0; y < cam.height; ++y) {
            std::memcpy(r.owned + static_cast<size_t>(y) * cam.width,
                        gray + static_cast<size_t>(y) * stride, cam.width);
        }
        lock.lock();
        r.frame = r.owned;
        r.stride = cam.width;
    }
    const int64_t ticket = s->next_ticket++;
    s->requests.emplace(ticket, std::move(r));
    s->pending[camera].push_back(ticket);
    ++s->submitted;
    lock.unlock();
    s->work_cv.notify_one();
    return ticket;
}

int32_t bd_server_wait(bd_server* s, int64_t ticket, bd_detection* out, int32_t* found,
                       double* latency_ms) {
    return collect(s, ticket, true, out, found, latency_ms);
}

int32_t bd_server_poll(bd_server* s, int64_t ticket, bd_detection* out, int32_t* found,
                       double* latency_ms) {
    return collect(s, ticket, false, out, found, latency_ms);
}

int32_t bd_server_get_stats(bd_server* s, bd_server_stats* out) {
    if (!s || !out) return BD_ERROR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lock(s->mutex);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->rejected = s->rejected;
    out->batches = s->batches;
    out->mean_batch_frames = s->batches ? static_cast<double>(s->batched_frames) / s->batches : 0.0;
    out->plans = static_cast<int32_t>(s->plans.size());
    out->peak_inflight = s->peak_inflight;
    out->device_bytes = s->device_bytes;
    return BD_OK;
}

}  // extern "C"
