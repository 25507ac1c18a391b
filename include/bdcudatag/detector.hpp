// bdcudatag C++ API (reference detector/include/bdcudatag/detector.hpp).
//
// Value types and an RAII detector over the C ABI in bdcudatag.h.  The class
// name, members, defaults and exceptions are those of the reference API, so
// C++ callers recompile against this header unchanged.  Calls on one
// Detector are serialised internally; sharing one between threads is safe
// but does not run frames in parallel.
#pragma once

#include <array>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "bdcudatag/bdcudatag.h"

namespace bdcudatag {

enum class Family : int32_t {
    Tag36h11 = BD_FAMILY_TAG36H11,
    Tag16h5 = BD_FAMILY_TAG16H5,
};

// Defaults match bd_config_init() (reference detector.hpp:23-33).
struct DetectorConfig {
    int max_hamming = -1;          // < 0: family default (tag36h11 2, tag16h5 1)
    int min_cluster_pixels = 24;   // smallest connected component considered
    int min_tag_pixels = 8;        // smallest bounding-box side considered
    int max_detections = 64;       // clamped to [1, 256]
    int max_candidates = 0;        // 0: derived from the frame area
    bool refine_edges = true;      // sub-pixel edge-line refinement
    bool use_cuda_graph = true;    // replay the host-frame pipeline as a CUDA graph
    float min_decision_margin = 3.0f;
    float decode_sharpening = 0.25f;
};

struct Detection {
    int id = -1;
    int hamming = 0;
    float decision_margin = 0.0f;
    // Top-left, top-right, bottom-right, bottom-left in the tag's canonical
    // orientation, pixel-index coordinates.
    std::array<std::array<float, 2>, 4> corners{};
    // Row-major map from the tag frame [-1, 1]^2 (x right, y down) to
    // pixels, scaled so homography[8] == 1.
    std::array<float, 9> homography{};

    float center_x() const {
        return 0.25f * (corners[0][0] + corners[1][0] + corners[2][0] + corners[3][0]);
    }
    float center_y() const {
        return 0.25f * (corners[0][1] + corners[1][1] + corners[2][1] + corners[3][1]);
    }
};

struct Stats {
    uint64_t frames = 0;
    float last_gpu_ms = 0.0f;
    float average_gpu_ms = 0.0f;
    float last_total_ms = 0.0f;
    int runs = 0;
    int candidates = 0;
    int detections = 0;
    int quads = 0;
    int roi_rows = 0;
};

class BD_API Detector {
public:
    Detector(Family family, int width, int height, const DetectorConfig& config = {});
    ~Detector();

    Detector(Detector&& other) noexcept;
    Detector& operator=(Detector&& other) noexcept;
    Detector(const Detector&) = delete;
    Detector& operator=(const Detector&) = delete;

    // Writes at most out_capacity detections; returns how many were written.
    int detect(const uint8_t* gray, int stride, Detection* out, int out_capacity);

    // Returns all detections in a new vector.
    std::vector<Detection> detect(const uint8_t* gray, int stride);

    // gray_device is a CUDA device pointer; no host-to-device copy is made.
    int detectDevice(const uint8_t* gray_device, int stride, Detection* out, int out_capacity);

    Stats stats() const;

    Family family() const { return family_; }
    int width() const { return width_; }
    int height() const { return height_; }

private:
    struct Impl;
    Impl* impl_ = nullptr;
    Family family_;
    int width_;
    int height_;
};

}  // namespace bdcudatag
