// C ABI and C++ API of bdcudatag on GB300.
//
// The fourteen reference symbols keep the reference's argument checks,
// error messages, status codes, return values and statistics
// (reference detector/src/detector.cpp:69-382, gpu_detector.cu:2100-2269);
// detection itself runs on a one-frame batch Plan (engine.cu).  The batch
// entry points of bdcudatag_gb300.h are new.

#include <algorithm>
#include <chrono>
#include <iterator>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "bdcudatag/bdcudatag.h"
#include "bdcudatag/bdcudatag_gb300.h"
#include "bdcudatag/detector.hpp"
#include "engine.h"
#include "pipeline.cuh"

namespace {

thread_local std::string g_last_error;

void set_error(const std::string& message) { g_last_error = message; }

struct FamilyInfo {
    const char* name;
    int bits_per_side;
    int min_hamming;
};

const FamilyInfo kFamilies[2] = {{"tag36h11", 6, 11}, {"tag16h5", 4, 5}};

bool valid_family(int family) { return family >= 0 && family < 2; }

bool valid_dimensions(int width, int height) {
    return width >= 16 && width <= BD_MAX_WIDTH && height >= 16 && height <= BD_MAX_HEIGHT;
}

int family_default_hamming(int family) { return family == BD_FAMILY_TAG36H11 ? 2 : 1; }

bool config_size_ok(const bd_config* config) {
    return !(config && config->struct_size != 0 && config->struct_size < sizeof(bd_config));
}

}  // namespace

namespace bdgb {
// Lets other translation units (noalloc.cu) report through bd_last_error().
void set_last_error(const char* message) { set_error(message ? message : ""); }
}  // namespace bdgb

struct bd_detector {
    bdgb::Plan* plan = nullptr;
    int family = 0;
    int width = 0;
    int height = 0;
    int max_detections = 0;
    int max_candidates = 0;
    // statistics (reference gpu_detector.cu:1829-1837)
    uint64_t frames = 0;
    float last_gpu_ms = 0.0f;
    float average_gpu_ms = 0.0f;
    float last_total_ms = 0.0f;
    int last_candidates = 0;
    int last_runs = 0;
    int last_detections = 0;
    int last_quads = 0;
    int last_roi_rows = 0;
};

struct bd_batch {
    bdgb::Plan* plan = nullptr;
};

namespace {

using Clock = std::chrono::steady_clock;

// Copies results and updates statistics (reference Impl::finish
// gpu_detector.cu:2100-2127).  The homography is already filled on the GPU.
int finish(bd_detector* d, bd_detection* out, int out_capacity, float total_ms) {
    const bdgb::Plan& plan = *d->plan;
    const bdgb::FrameResultHeader* hdr = plan.result(0);
    const int found = std::min(static_cast<int>(hdr->found[d->family]), d->max_detections);
    const int written = std::min(found, std::max(out_capacity, 0));
    if (written > 0 && out) {
        std::memcpy(out, plan.detections(0, d->family), static_cast<size_t>(written) * sizeof(bd_detection));
    }
    d->last_candidates = std::min(static_cast<int>(hdr->counts[0]), d->max_candidates);
    d->last_runs = static_cast<int>(hdr->counts[2]);
    d->last_detections = found;
    d->last_quads = static_cast<int>(hdr->counts[3]);
    d->last_roi_rows = std::min(static_cast<int>(hdr->counts[4]) * bdgb::kTile, d->height);
    const float gpu_ms = plan.last_gpu_ms();
    d->last_gpu_ms = gpu_ms;
    d->last_total_ms = total_ms;
    d->average_gpu_ms = d->frames == 0 ? gpu_ms : 0.9f * d->average_gpu_ms + 0.1f * gpu_ms;
    ++d->frames;
    return found;
}

int check_detect_args(bd_detector* detector, const uint8_t* gray, int32_t stride, bd_detection* out,
                      int32_t out_capacity, const char* null_message) {
    if (!detector) {
        set_error("null detector");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (!gray) {
        set_error(null_message);
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (stride < detector->width) {
        set_error("stride is smaller than the image width");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (out_capacity < 0 || (out_capacity > 0 && !out)) {
        set_error("invalid output buffer");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    return BD_OK;
}

int32_t detect_common(bd_detector* detector, const uint8_t* gray, int32_t stride, bd_detection* out,
                      int32_t out_capacity, bool device) {
    const int bad = check_detect_args(detector, gray, stride, out, out_capacity,
                                      device ? "null device image pointer" : "null image pointer");
    if (bad != BD_OK) return bad;
    bdgb::Plan& plan = *detector->plan;
    const std::lock_guard<std::mutex> lock(plan.mutex());
    const auto start = Clock::now();
    std::string error;
    const uint8_t* frames[1] = {gray};
    const int32_t strides[1] = {stride};
    const int rc = device ? plan.run_device(frames, strides, &error) : plan.run_host(frames, strides, &error);
    if (rc != 0) {
        set_error(error.empty() ? "CUDA detection failed" : error);
        return BD_ERROR_CUDA;
    }
    const float total_ms = std::chrono::duration<float, std::milli>(Clock::now() - start).count();
    return finish(detector, out, out_capacity, total_ms);
}

int32_t batch_collect(bd_batch* batch, bd_detection* out, int32_t* found) {
    const bdgb::Plan& plan = *batch->plan;
    const int md = plan.max_detections();
    for (int i = 0; i < plan.frames(); ++i) {
        for (int f = 0; f < 2; ++f) {
            const bool on = (plan.frame(i).families >> f) & 1u;
            const int n = on ? std::min(plan.found(i, f), md) : -1;
            if (found) found[2 * i + f] = n;
            if (out && n > 0) {
                std::memcpy(out + (static_cast<size_t>(i) * 2 + f) * md, plan.detections(i, f),
                            static_cast<size_t>(n) * sizeof(bd_detection));
            }
        }
    }
    return BD_OK;
}

int32_t batch_check(bd_batch* batch, const uint8_t* const* frames, const int32_t* strides) {
    if (!batch) {
        set_error("null batch");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (!frames || !strides) {
        set_error("null frame or stride array");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    for (int i = 0; i < batch->plan->frames(); ++i) {
        if (!frames[i]) {
            set_error("null image pointer");
            return BD_ERROR_INVALID_ARGUMENT;
        }
        if (strides[i] < batch->plan->frame(i).width) {
            set_error("stride is smaller than the image width");
            return BD_ERROR_INVALID_ARGUMENT;
        }
    }
    return BD_OK;
}

}  // namespace

extern "C" {

uint32_t bd_api_version(void) { return BD_API_VERSION; }

const char* bd_version_string(void) { return "bdcudatag 0.1.0"; }

int32_t bd_family_count(void) { return 2; }

const char* bd_family_name(int32_t family) {
    if (!valid_family(family)) return nullptr;
    return kFamilies[family].name;
}

int32_t bd_family_bits_per_side(int32_t family) {
    if (!valid_family(family)) return -1;
    return kFamilies[family].bits_per_side;
}

int32_t bd_family_min_hamming(int32_t family) {
    if (!valid_family(family)) return -1;
    return kFamilies[family].min_hamming;
}

int32_t bd_family_default_max_hamming(int32_t family) {
    if (!valid_family(family)) return -1;
    return family_default_hamming(family);
}

void bd_config_init(bd_config* config) {
    if (!config) return;
    std::memset(config, 0, sizeof(*config));
    config->struct_size = sizeof(bd_config);
    config->max_hamming = -1;
    config->min_cluster_pixels = 24;
    config->min_tag_pixels = 8;
    config->max_detections = 64;
    config->max_candidates = 0;
    config->refine_edges = 1;
    config->use_cuda_graph = 1;
    config->min_decision_margin = 3.0f;
    config->decode_sharpening = 0.25f;
}

bd_detector* bd_detector_create(int32_t family, int32_t width, int32_t height,
                                const bd_config* config, int32_t* status_out) {
    if (status_out) *status_out = BD_OK;
    if (!valid_family(family)) {
        set_error("unknown tag family");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    if (!valid_dimensions(width, height)) {
        set_error("image dimensions out of range (16..8192 x 16..16384)");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    if (!config_size_ok(config)) {
        set_error("bd_config.struct_size is too small for this library version");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    const bdgb::PlanConfig pc = bdgb::resolve_config(config);
    bdgb::PlanFrame frame;
    frame.width = width;
    frame.height = height;
    frame.families = 1u << family;
    std::string error;
    bdgb::Plan* plan = bdgb::Plan::create({frame}, pc, &error);
    if (!plan) {
        set_error(error.empty() ? "failed to create CUDA detector" : error);
        if (status_out) *status_out = BD_ERROR_CUDA;
        return nullptr;
    }
    bd_detector* detector = new (std::nothrow) bd_detector();
    if (!detector) {
        delete plan;
        set_error("out of memory allocating detector handle");
        if (status_out) *status_out = BD_ERROR_OUT_OF_MEMORY;
        return nullptr;
    }
    detector->plan = plan;
    detector->family = family;
    detector->width = width;
    detector->height = height;
    detector->max_detections = pc.max_detections;
    detector->max_candidates = plan->max_candidates(0);
    return detector;
}

void bd_detector_destroy(bd_detector* detector) {
    if (!detector) return;
    delete detector->plan;
    delete detector;
}

int32_t bd_detector_detect_host(bd_detector* detector, const uint8_t* gray, int32_t stride,
                                bd_detection* out, int32_t out_capacity) {
    return detect_common(detector, gray, stride, out, out_capacity, false);
}

int32_t bd_detector_detect_device(bd_detector* detector, const uint8_t* gray_device,
                                  int32_t stride, bd_detection* out, int32_t out_capacity) {
    return detect_common(detector, gray_device, stride, out, out_capacity, true);
}

void bd_detector_get_stats(bd_detector* detector, bd_stats* out) {
    if (!detector || !out) return;
    const std::lock_guard<std::mutex> lock(detector->plan->mutex());
    out->frames = detector->frames;
    out->last_gpu_ms = detector->last_gpu_ms;
    out->average_gpu_ms = detector->average_gpu_ms;
    out->last_total_ms = detector->last_total_ms;
    out->runs = detector->last_runs;
    out->candidates = detector->last_candidates;
    out->detections = detector->last_detections;
    out->quads = detector->last_quads;
    out->roi_rows = detector->last_roi_rows;
}

const char* bd_last_error(void) { return g_last_error.c_str(); }

// --- batches ------------------------------------------------------------------

bd_batch* bd_batch_create(const bd_camera* cameras, int32_t count, const bd_config* config,
                          int32_t* status_out) {
    if (status_out) *status_out = BD_OK;
    if (!cameras || count < 1 || count > BD_BATCH_MAX_CAMERAS) {
        set_error("a batch needs 1 to 64 cameras");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    if (!config_size_ok(config)) {
        set_error("bd_config.struct_size is too small for this library version");
        if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
        return nullptr;
    }
    std::vector<bdgb::PlanFrame> frames(count);
    for (int i = 0; i < count; ++i) {
        if (!valid_dimensions(cameras[i].width, cameras[i].height)) {
            set_error("image dimensions out of range (16..8192 x 16..16384)");
            if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
            return nullptr;
        }
        if ((cameras[i].families & 3u) == 0 || (cameras[i].families & ~3u) != 0) {
            set_error("camera family mask must select tag36h11 and/or tag16h5");
            if (status_out) *status_out = BD_ERROR_INVALID_ARGUMENT;
            return nullptr;
        }
        frames[i].width = cameras[i].width;
        frames[i].height = cameras[i].height;
        frames[i].families = cameras[i].families;
    }
    std::string error;
    bdgb::Plan* plan = bdgb::Plan::create(frames, bdgb::resolve_config(config), &error);
    if (!plan) {
        set_error(error.empty() ? "failed to create CUDA batch" : error);
        if (status_out) *status_out = BD_ERROR_CUDA;
        return nullptr;
    }
    bd_batch* batch = new (std::nothrow) bd_batch();
    if (!batch) {
        delete plan;
        set_error("out of memory allocating batch handle");
        if (status_out) *status_out = BD_ERROR_OUT_OF_MEMORY;
        return nullptr;
    }
    batch->plan = plan;
    return batch;
}

void bd_batch_destroy(bd_batch* batch) {
    if (!batch) return;
    delete batch->plan;
    delete batch;
}

int32_t bd_batch_camera_count(const bd_batch* batch) { return batch ? batch->plan->frames() : 0; }

int32_t bd_batch_max_detections(const bd_batch* batch) {
    return batch ? batch->plan->max_detections() : 0;
}

int64_t bd_batch_device_bytes(const bd_batch* batch) {
    return batch ? static_cast<int64_t>(batch->plan->device_bytes()) : 0;
}

int32_t bd_batch_submit_host(bd_batch* batch, const uint8_t* const* frames, const int32_t* strides) {
    const int bad = batch_check(batch, frames, strides);
    if (bad != BD_OK) return bad;
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->submit_host(frames, strides, &error) != 0) {
        set_error(error);
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}

int32_t bd_batch_submit_device(bd_batch* batch, const uint8_t* const* frames,
                               const int32_t* strides) {
    const int bad = batch_check(batch, frames, strides);
    if (bad != BD_OK) return bad;
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->submit_device(frames, strides, &error) != 0) {
        set_error(error);
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}

int32_t bd_batch_wait(bd_batch* batch, bd_detection* out, int32_t* found) {
    if (!batch) {
        set_error("null batch");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->wait(&error) != 0) {
        set_error(error);
        return BD_ERROR_CUDA;
    }
    return batch_collect(batch, out, found);
}

int32_t bd_batch_query(bd_batch* batch) {
    if (!batch) {
        set_error("null batch");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    const int r = batch->plan->query(&error);
    if (r < 0) {
        set_error(error);
        return BD_ERROR_CUDA;
    }
    return r;
}

int32_t bd_batch_detect_host(bd_batch* batch, const uint8_t* const* frames, const int32_t* strides,
                             bd_detection* out, int32_t* found) {
    const int rc = bd_batch_submit_host(batch, frames, strides);
    if (rc != BD_OK) return rc;
    return bd_batch_wait(batch, out, found);
}

int32_t bd_batch_detect_device(bd_batch* batch, const uint8_t* const* frames,
                               const int32_t* strides, bd_detection* out, int32_t* found) {
    const int rc = bd_batch_submit_device(batch, frames, strides);
    if (rc != BD_OK) return rc;
    return bd_batch_wait(batch, out, found);
}

int32_t bd_batch_pipeline(bd_batch* const* batches, int32_t count, const uint8_t* const* frames,
                          const int32_t* strides, int32_t sets, int32_t steps, int32_t device,
                          float* latency_ms, double* wall_ms) {
    if (!batches || count < 1 || !frames || !strides || sets < 1 || steps < 0) {
        set_error("bd_batch_pipeline: bad arguments");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const int cams = batches[0] ? batches[0]->plan->frames() : 0;
    for (int i = 0; i < count; ++i) {
        bool same = batches[i] && batches[i]->plan->frames() == cams;
        for (int c = 0; same && c < cams; ++c) {
            const bdgb::PlanFrame& a = batches[i]->plan->frame(c);
            const bdgb::PlanFrame& b0 = batches[0]->plan->frame(c);
            same = a.width == b0.width && a.height == b0.height && a.families == b0.families;
        }
        for (int j = 0; same && j < i; ++j) same = batches[j] != batches[i];
        if (!same) {
            set_error("bd_batch_pipeline: batches must be distinct, non-null, with the same cameras");
            return BD_ERROR_INVALID_ARGUMENT;
        }
    }
    for (int k = 0; k < sets; ++k) {
        const int bad = batch_check(batches[0], frames + static_cast<size_t>(k) * cams, strides);
        if (bad != BD_OK) return bad;
    }
    // Each batch is used by this call alone while it runs; the mutexes are
    // taken in address order so concurrent callers cannot deadlock.
    std::vector<std::mutex*> order;
    for (int i = 0; i < count; ++i) order.push_back(&batches[i]->plan->mutex());
    std::sort(order.begin(), order.end());
    std::vector<std::unique_lock<std::mutex>> locks;
    locks.reserve(count);
    for (std::mutex* m : order) locks.emplace_back(*m);
    std::vector<bool> busy(count, false);
    std::vector<int> step_of(count, -1);
    std::vector<Clock::time_point> issued(count);
    std::string error;
    auto finish_one = [&](int i) -> bool {
        bdgb::Plan& plan = *batches[i]->plan;
        if (plan.wait(&error) != 0) return false;
        if (latency_ms) {
            latency_ms[step_of[i]] =
                std::chrono::duration<float, std::milli>(Clock::now() - issued[i]).count();
        }
        busy[i] = false;
        return true;
    };
    const auto t0 = Clock::now();
    for (int k = 0; k < steps; ++k) {
        const int i = k % count;
        while (busy[i]) {
            // Poll every batch in flight so completions are stamped on time.
            for (int j = 0; j < count; ++j) {
                if (!busy[j]) continue;
                const int q = batches[j]->plan->query(&error);
                if (q < 0 || (q == 1 && !finish_one(j))) {
                    set_error(error);
                    return BD_ERROR_CUDA;
                }
            }
        }
        const uint8_t* const* set = frames + static_cast<size_t>(k % sets) * cams;
        issued[i] = Clock::now();
        step_of[i] = k;
        bdgb::Plan& plan = *batches[i]->plan;
        const int rc = device ? plan.submit_device(set, strides, &error)
                              : plan.submit_host(set, strides, &error);
        if (rc != 0) {
            set_error(error);
            return BD_ERROR_CUDA;
        }
        busy[i] = true;
    }
    for (int i = 0; i < count; ++i) {
        while (busy[i]) {
            for (int j = 0; j < count; ++j) {
                if (!busy[j]) continue;
                const int q = batches[j]->plan->query(&error);
                if (q < 0 || (q == 1 && !finish_one(j))) {
                    set_error(error);
                    return BD_ERROR_CUDA;
                }
            }
        }
    }
    if (wall_ms) *wall_ms = std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
    return BD_OK;
}

int32_t bd_batch_set_stream(bd_batch* batch, void* cuda_stream) {
    if (!batch) {
        set_error("null batch");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    batch->plan->set_stream(cuda_stream);
    return BD_OK;
}

int32_t bd_batch_get_launch(const bd_batch* batch, bd_launch_config* out) {
    if (!batch || !out) return BD_ERROR_INVALID_ARGUMENT;
    const bdgb::LaunchConfig& lc = batch->plan->launch();
    out->stats_rows = lc.stats_rows;
    out->quad_warps = lc.quad_warps;
    out->quad_ctas_per_sm = lc.quad_ctas_per_sm;
    out->quad_split = lc.quad_split;
    out->band_cap = lc.band_cap;
    out->fit_merged = lc.fit_merged;
    out->persistent = lc.persistent;
    out->persist_ctas = lc.persist_ctas;
    return BD_OK;
}

int32_t bd_batch_set_launch(bd_batch* batch, const bd_launch_config* launch) {
    if (!batch || !launch) {
        set_error("null batch or launch config");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    bdgb::LaunchConfig lc;
    lc.stats_rows = launch->stats_rows;
    lc.quad_warps = launch->quad_warps;
    lc.quad_ctas_per_sm = launch->quad_ctas_per_sm;
    lc.quad_split = launch->quad_split;
    lc.band_cap = launch->band_cap;
    lc.fit_merged = launch->fit_merged;
    lc.persistent = launch->persistent;
    lc.persist_ctas = launch->persist_ctas;
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->set_launch(lc, &error) != 0) {
        set_error(error);
        return error.rfind("launch config", 0) == 0 ? BD_ERROR_INVALID_ARGUMENT : BD_ERROR_CUDA;
    }
    return BD_OK;
}

int32_t bd_batch_autotune(bd_batch* batch, const uint8_t* const* frames_device,
                          const int32_t* strides, int32_t iterations, bd_launch_config* best_out,
                          float* best_ms_out) {
    const int bad = batch_check(batch, frames_device, strides);
    if (bad != BD_OK) return bad;
    std::string error;
    float ms = 0.0f;
    {
        const std::lock_guard<std::mutex> lock(batch->plan->mutex());
        if (batch->plan->autotune(frames_device, strides, iterations, &ms, &error) != 0) {
            set_error(error);
            return BD_ERROR_CUDA;
        }
    }
    if (best_out) bd_batch_get_launch(batch, best_out);
    if (best_ms_out) *best_ms_out = ms;
    return BD_OK;
}

int32_t bd_batch_debug_persist(bd_batch* batch, int64_t timeout_ns, int32_t stall_frame) {
    if (!batch) {
        set_error("null batch");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->set_persist_params(timeout_ns, stall_frame, &error) != 0) {
        set_error(error);
        return BD_ERROR_INVALID_ARGUMENT;
    }
    return BD_OK;
}

int32_t bd_stage_count(void) { return bdgb::kStageCount; }

const char* bd_stage_name(int32_t stage) {
    if (stage < 0 || stage >= bdgb::kStageCount) return nullptr;
    return bdgb::kStageNames[stage];
}

int32_t bd_batch_profile_device(bd_batch* batch, const uint8_t* const* frames,
                                const int32_t* strides, float* stage_ms) {
    const int bad = batch_check(batch, frames, strides);
    if (bad != BD_OK) return bad;
    if (!stage_ms) {
        set_error("null stage time array");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    std::string error;
    if (batch->plan->profile_device(frames, strides, stage_ms, &error) != 0) {
        set_error(error);
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}

uint8_t* bd_batch_host_frame(bd_batch* batch, int32_t camera) {
    if (!batch || camera < 0 || camera >= batch->plan->frames()) return nullptr;
    return batch->plan->host_frame(camera);
}

float bd_batch_last_gpu_ms(const bd_batch* batch) { return batch ? batch->plan->last_gpu_ms() : 0.0f; }

int32_t bd_batch_counts(const bd_batch* batch, int32_t camera, uint32_t counts[5]) {
    if (!batch || !counts || camera < 0 || camera >= batch->plan->frames()) {
        return BD_ERROR_INVALID_ARGUMENT;
    }
    std::memcpy(counts, batch->plan->result(camera)->counts, 5 * sizeof(uint32_t));
    return BD_OK;
}

int64_t bd_batch_debug_stage(bd_batch* batch, int32_t camera, const char* name, void* dst,
                             int64_t dst_bytes) {
    if (!batch) return -1;
    const std::lock_guard<std::mutex> lock(batch->plan->mutex());
    return batch->plan->copy_stage(camera, name, dst, dst_bytes);
}

int64_t bd_detector_debug_stage(bd_detector* detector, const char* name, void* dst,
                                int64_t dst_bytes) {
    if (!detector) return -1;
    const std::lock_guard<std::mutex> lock(detector->plan->mutex());
    return detector->plan->copy_stage(0, name, dst, dst_bytes);
}

}  // extern "C"

// --- C++ API --------------------------------------------------------------------
//
// bdcudatag::Detector (include/bdcudatag/detector.hpp, the reference's public
// C++ API) over the C ABI above.  The behaviour the API fixes is kept: the
// exception types and texts callers may match on, the clamp of the output
// capacity to max_detections, and a lock that serialises calls on one object
// (reference detector.cpp:229-382).  Here the owned state is one RAII object:
// the C handle lives and dies with Impl, so the Detector's special members
// only move or delete that object.

namespace bdcudatag {

namespace {

constexpr const char* kMovedFrom = "detector has been moved from";

bd_config to_native(const DetectorConfig& c) {
    bd_config n;
    bd_config_init(&n);
    n.max_hamming = c.max_hamming;
    n.min_cluster_pixels = c.min_cluster_pixels;
    n.min_tag_pixels = c.min_tag_pixels;
    n.max_detections = c.max_detections;
    n.max_candidates = c.max_candidates;
    n.refine_edges = c.refine_edges ? 1 : 0;
    n.use_cuda_graph = c.use_cuda_graph ? 1 : 0;
    n.min_decision_margin = c.min_decision_margin;
    n.decode_sharpening = c.decode_sharpening;
    return n;
}

Detection from_native(const bd_detection& r) {
    Detection d;
    d.id = r.id;
    d.hamming = r.hamming;
    d.decision_margin = r.decision_margin;
    for (size_t k = 0; k < d.corners.size(); ++k) d.corners[k] = {r.corners[2 * k], r.corners[2 * k + 1]};
    std::copy(std::begin(r.homography), std::end(r.homography), d.homography.begin());
    return d;
}

Stats from_native(const bd_stats& s) {
    Stats o;
    o.frames = s.frames;
    o.last_gpu_ms = s.last_gpu_ms;
    o.average_gpu_ms = s.average_gpu_ms;
    o.last_total_ms = s.last_total_ms;
    o.runs = s.runs;
    o.candidates = s.candidates;
    o.detections = s.detections;
    o.quads = s.quads;
    o.roi_rows = s.roi_rows;
    return o;
}

using DetectFn = int32_t (*)(bd_detector*, const uint8_t*, int32_t, bd_detection*, int32_t);

}  // namespace

// The C detector plus the record buffer its results land in before they are
// converted; the lock covers both.
struct Detector::Impl {
    bd_detector* handle = nullptr;
    std::vector<bd_detection> records;
    mutable std::mutex lock;

    Impl(Family family, int width, int height, const DetectorConfig& config) {
        const bd_config native = to_native(config);
        int32_t status = BD_OK;
        handle = bd_detector_create(static_cast<int32_t>(family), width, height, &native, &status);
        if (!handle) {
            const std::string why = bd_last_error();
            throw std::runtime_error(why.empty() ? "failed to create bdcudatag detector" : why);
        }
        records.resize(static_cast<size_t>(std::clamp(native.max_detections, 1, 256)));
    }
    ~Impl() { bd_detector_destroy(handle); }
    Impl(const Impl&) = delete;
    Impl& operator=(const Impl&) = delete;

    int capacity() const { return static_cast<int>(records.size()); }

    // One call of the host or device entry point; converts what was written.
    int run(DetectFn fn, const uint8_t* image, int stride, Detection* out, int out_capacity) {
        if (out_capacity < 0 || (out_capacity > 0 && !out)) {
            throw std::invalid_argument("invalid detection output buffer");
        }
        const int cap = std::min(out_capacity, capacity());
        const std::lock_guard<std::mutex> hold(lock);
        const int found = fn(handle, image, stride, records.data(), cap);
        if (found < 0) throw std::runtime_error(bd_last_error());
        const int written = std::min(found, cap);
        std::transform(records.begin(), records.begin() + written, out,
                       [](const bd_detection& r) { return from_native(r); });
        return written;
    }
};

Detector::Detector(Family family, int width, int height, const DetectorConfig& config)
    : impl_(new Impl(family, width, height, config)), family_(family), width_(width),
      height_(height) {}

Detector::~Detector() { delete impl_; }

Detector::Detector(Detector&& other) noexcept
    : impl_(std::exchange(other.impl_, nullptr)), family_(other.family_), width_(other.width_),
      height_(other.height_) {}

Detector& Detector::operator=(Detector&& other) noexcept {
    if (this != &other) {
        delete std::exchange(impl_, std::exchange(other.impl_, nullptr));
        family_ = other.family_;
        width_ = other.width_;
        height_ = other.height_;
    }
    return *this;
}

int Detector::detect(const uint8_t* gray, int stride, Detection* out, int out_capacity) {
    if (!impl_) throw std::runtime_error(kMovedFrom);
    return impl_->run(&bd_detector_detect_host, gray, stride, out, out_capacity);
}

std::vector<Detection> Detector::detect(const uint8_t* gray, int stride) {
    if (!impl_) throw std::runtime_error(kMovedFrom);
    std::vector<Detection> all(static_cast<size_t>(impl_->capacity()));
    all.resize(static_cast<size_t>(impl_->run(&bd_detector_detect_host, gray, stride, all.data(),
                                              impl_->capacity())));
    return all;
}

int Detector::detectDevice(const uint8_t* gray_device, int stride, Detection* out, int out_capacity) {
    if (!impl_) throw std::runtime_error(kMovedFrom);
    return impl_->run(&bd_detector_detect_device, gray_device, stride, out, out_capacity);
}

Stats Detector::stats() const {
    if (!impl_) return {};
    bd_stats native;
    {
        const std::lock_guard<std::mutex> hold(impl_->lock);
        bd_detector_get_stats(impl_->handle, &native);
    }
    return from_native(native);
}

}  // namespace bdcudatag
