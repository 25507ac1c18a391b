// Host engine of the batched pipeline.  No CUDA types appear here, so the
// C ABI layer (capi.cpp) compiles with the host compiler alone.
#pragma once

#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "bdcudatag/bdcudatag.h"

namespace bdgb {

struct FrameResultHeader;
struct LaunchConfig;

struct PlanFrame {
    int width = 0;
    int height = 0;
    uint32_t families = 1;  // bit f: decode family f (0 tag36h11, 1 tag16h5)
};

// Resolved settings shared by every frame of a plan (clamping as
// reference gpu_detector.cu:1905-1943).
struct PlanConfig {
    int max_hamming[2] = {2, 1};
    int min_cluster_pixels = 24;
    int min_tag_pixels = 8;
    int max_detections = 64;
    int max_candidates = 0;       // 0: per frame, from the frame area
    bool refine_edges = true;
    bool use_graph = true;
    float min_decision_margin = 3.0f;
    float decode_sharpening = 0.25f;
};

// Resolves a bd_config (NULL: defaults) for the given family set.
PlanConfig resolve_config(const bd_config* config);
int auto_max_candidates(int width, int height, int configured);

class Plan {
public:
    // Returns nullptr and fills *error on failure.
    static Plan* create(const std::vector<PlanFrame>& frames, const PlanConfig& config,
                        std::string* error);
    ~Plan();
    Plan(const Plan&) = delete;
    Plan& operator=(const Plan&) = delete;

    // Synchronous batch: frames[i] / strides[i] for every frame of the plan.
    // Host frames are copied into pinned staging first.  Returns 0 or -1.
    int run_host(const uint8_t* const* frames, const int32_t* strides, std::string* error);
    int run_device(const uint8_t* const* frames, const int32_t* strides, std::string* error);

    // Asynchronous halves of run_*: enqueue, then wait for the results.
    int submit_host(const uint8_t* const* frames, const int32_t* strides, std::string* error);
    int submit_device(const uint8_t* const* frames, const int32_t* strides, std::string* error);
    int wait(std::string* error);
    // 1: nothing in flight or finished; 0: running; -1: error.
    int query(std::string* error);

    // Batch with some slots unused: frames[i] == nullptr leaves slot i out
    // of this launch (its kernels return at once and it reports nothing).
    // Host frames (page-locked or not) are copied to the plan's device
    // buffers; results as for submit_host.
    int submit_slots(const uint8_t* const* frames, const int32_t* strides, std::string* error);

    // Launch shapes (results do not depend on them).  set_launch re-captures
    // the graphs; autotune times candidate shapes on `iterations` device-input
    // runs of `frames` (coordinate descent) and keeps the fastest.
    int set_launch(const LaunchConfig& launch, std::string* error);
    const LaunchConfig& launch() const;
    int autotune(const uint8_t* const* frames, const int32_t* strides, int iterations,
                 float* best_ms, std::string* error);

    // Test hook of the persistent launch: the queue-wait limit, and a frame
    // (-1: none) one of whose items is withheld so that the wait runs out.
    int set_persist_params(int64_t timeout_ns, int stall_frame, std::string* error);

    // Stream for later submits (a cudaStream_t; null: the plan's own).
    void set_stream(void* stream);

    // One synchronous device-input run, not graphed, with CUDA events
    // around every kernel; writes kStageCount stage times (ms).
    int profile_device(const uint8_t* const* frames, const int32_t* strides, float* stage_ms,
                       std::string* error);

    // Results of the last completed run (host memory).
    const FrameResultHeader* result(int frame) const;
    const bd_detection* detections(int frame, int family) const;
    int found(int frame, int family) const;
    float last_gpu_ms() const { return last_gpu_ms_; }

    int frames() const { return static_cast<int>(frames_.size()); }
    int max_detections() const { return config_.max_detections; }
    int max_candidates(int frame) const;
    const PlanFrame& frame(int i) const { return frames_[i]; }
    size_t device_bytes() const { return arena_bytes_; }

    // Copies a named per-frame device buffer (test hook; see capi).
    int64_t copy_stage(int frame, const char* name, void* dst, int64_t dst_bytes);

    // Serialises users of one plan (the C ABI holds it around a call).
    std::mutex& mutex() { return mutex_; }

    // The pinned staging buffer of frame i (width*height bytes), for callers
    // that render straight into it.
    uint8_t* host_frame(int i);

private:
    Plan() = default;
    struct Impl;
    Impl* impl_ = nullptr;
    std::vector<PlanFrame> frames_;
    PlanConfig config_;
    size_t arena_bytes_ = 0;
    float last_gpu_ms_ = 0.0f;
    std::mutex mutex_;
    friend struct PlanAccess;
};

}  // namespace bdgb
