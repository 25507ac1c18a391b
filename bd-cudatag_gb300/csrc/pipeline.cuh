// Shared layout of the batched detection pipeline: per-frame descriptors,
// per-frame device state and result records.  Included by the kernels
// (k_front.cu, k_quad.cu, k_finalize.cu) and the host engine (engine.cu).
//
// One launch of each stage covers every frame of a batch.  A frame is cut
// into "bands" of 8 pixel rows (one tile row); stages 1-6 run one CTA per
// band, so a batch of frames of any mix of sizes is one flat grid whose CTAs
// find their frame by binary search over a prefix of band counts.
#pragma once

#include <stdint.h>

#include "bdcudatag/bdcudatag.h"

#if defined(__CUDACC__)
#define BDGB_HD __host__ __device__
#else
#define BDGB_HD
#endif

namespace bdgb {

constexpr int kMaxFrames = 64;         // frames in one batch plan
constexpr int kMaxBandsPerFrame = BD_MAX_HEIGHT / 8;  // 8-row bands of the tallest frame
constexpr int kTile = 8;               // tile side, pixels
constexpr int kMinTileContrast = 12;   // reference gpu_detector.cu:39
constexpr int kFitDirections = 32;     // :46
constexpr int kMaxBoundaryRows = 1024; // :47
constexpr int kMaxHullVertices = 64;   // :48
constexpr int kFitIterations = 2;      // :49
constexpr int kFitProbeHalf = 24;      // :50
constexpr int kMaxDetectionsCap = 256;
constexpr uint32_t kNone = 0xffffffffu;

// Counters and per-frame reductions, zeroed at the start of every batch.
struct FrameState {
    uint32_t counts[5];      // [0] candidates (uncapped) [2] runs [3] quads [4] ROI tile rows
    uint32_t top_enc;        // tile_h - first active tile row (0: none)
    uint32_t bottom_enc;     // last active tile row + 1 (0: none)
    uint32_t ref[2];         // noise-floor span quartile, Otsu level
    uint32_t done_stats;     // stats units finished (the persistent launch)
    uint32_t done_cands;     // CTAs of the candidate-count stage finished
    uint32_t n_candidates;   // min(counts[0], max_candidates)
    uint32_t n_big;          // candidates above the big-candidate split (front of FrameDesc::fit_list)
    uint32_t n_small;        // the others (back of FrameDesc::fit_list)
    uint32_t span_hist[256];
    uint32_t mean_hist[64];
    uint32_t bin_base[64];   // first flattened position of each area bin
    // Units finished per stage, for the persistent launch (k_persistent.cu);
    // the per-stage launches use done_stats and done_cands only.
    uint32_t done_bin, done_merge, done_region, done_fit, done_final;
    uint32_t fit_units;      // fit units queued for this frame
    uint32_t small_next;     // next (small candidate, family) pair a warp takes
    // Frame 0 only: the next big candidate / small pair of the whole batch
    // that k_fit_decode_all hands out.
    uint32_t batch_big_next, batch_small_next;
    uint32_t pad_state[1];   // size a multiple of 16 bytes (the work queue follows the states)
};

// Work queue of one batch for the persistent launch: queue positions
// [0, seed) are the frames' tile-statistics units, implied by the batch
// descriptor; position seed + s is items[s], published by the CTA that
// finished the previous stage of a frame.  Zeroed with the frame states
// before every batch (0 = not yet published).
struct WorkQueue {
    uint32_t head;          // next position to claim
    uint32_t reserve;       // item slots reserved by pushes
    uint32_t frames_done;   // frames whose last finalize unit ended
    uint32_t finished;      // 1: every frame is done, or the launch gave up
    uint32_t status;        // 0, or kQueueTimeout / kQueueOverflow bits
    uint32_t pad[3];
    uint32_t items[1];      // `capacity` slots (the array runs on)
};
constexpr uint32_t kQueueTimeout = 1u;   // a wait for a queue slot ran out of time
constexpr uint32_t kQueueOverflow = 2u;  // more items than the queue holds (a bug)

// Item slots a frame can need (everything but its statistics units): four
// band stages, one fit unit per big candidate or eight (candidate, family)
// pairs, two finalize units.
BDGB_HD inline uint32_t queue_items_per_frame(int tile_h, int max_candidates) {
    return 4u * static_cast<uint32_t>(tile_h) + static_cast<uint32_t>(max_candidates) +
           static_cast<uint32_t>((2 * max_candidates + 7) / 8) + 2u;
}

// One decoded candidate (per family): id -1 when nothing decoded.
struct DecodeOut {
    int32_t id;
    int32_t hamming;
    float margin;
    float corners[8];
};

// Result header of one frame; followed by 2 * max_detections bd_detection
// records (family 0 block, then family 1 block).
struct FrameResultHeader {
    uint32_t counts[5];
    uint32_t found[2];       // detections per family after de-duplication
    uint32_t pad;
};

// Input of one frame for one call: device pointer and row stride.
struct FrameIO {
    const uint8_t* gray;
    int64_t stride;
};

struct FrameDesc {
    int32_t width, height;
    int32_t tile_w, tile_h, words, row_cap;
    int32_t max_candidates, max_detections;
    uint32_t families;             // bit f set: decode family f
    int32_t min_cluster_pixels, min_tag_pixels, refine_edges;
    int32_t max_hamming[2];
    float min_margin, sharpening;
    // device buffers of this frame
    uint8_t* tile_min;             // tile_w * tile_h
    uint8_t* tile_max;
    int32_t* row_lo;               // first / last contrasting tile per tile row (-1: none)
    int32_t* row_hi;
    uint32_t* bits;                // height * words, 1 = white
    uint32_t* row_count;           // height
    uint32_t* runs;                // slots (height * row_cap): x0 | x1 << 16
    uint32_t* parent;              // slots: union-find, then the root of every run
    uint32_t* area;                // slots (valid at roots)
    uint32_t* bbox;                // 4 * slots (valid at roots)
    uint32_t* cand_meta;           // slots: per band (at its first slot) bin << 24 | big << 23 |
                                   // rank in band of each candidate listed in lroots
    uint32_t* lroots;              // slots: per band (at its first slot) the band-local roots
    uint32_t* lroot_count;         // tile_h: band-local roots per band
    uint32_t* band_mode;           // tile_h: bit 0 fallback (one root per run), else bit r: row r
                                   // starts a shared-memory segment (band-local unions done)
    uint32_t* band_bins;           // tile_h * 64 candidate counts, then exclusive prefixes
    uint32_t* candidates;          // max_candidates root slots, canonical order
    uint32_t* fit_list;            // max_candidates positions in `candidates`: from the front the
                                   // n_big whose bbox side exceeds the split (k_fit_decode_big),
                                   // from the back the n_small others (k_fit_decode); any order
    FrameState* state;
    float* hull_quads;             // max_candidates * 8
    float* quads;                  // 2 * max_candidates * 8 (per family)
    DecodeOut* decodes;            // 2 * max_candidates
    FrameResultHeader* result;     // header + 2 * max_detections records
};

struct BatchDesc {
    int32_t frames;
    uint32_t queue_capacity;              // item slots of the batch's WorkQueue
    int32_t total_bands;
    int32_t band_prefix[kMaxFrames + 1];  // exclusive prefix of tile_h over frames
    int32_t stats_rows;                   // tile rows per k_stats CTA
    int32_t stats_ctas;
    int32_t stats_prefix[kMaxFrames + 1]; // exclusive prefix of ceil(tile_h / stats_rows)
    FrameDesc f[kMaxFrames];
};

// Launch shapes that do not change any result (tuned per plan).
constexpr int kMaxQuadWarps = 8;
struct LaunchConfig {
    int stats_rows = 1;        // tile rows per k_stats CTA: 1, 2 or 4
    int quad_warps = 4;        // warps (= candidates in flight) per k_fit_decode CTA: 2, 4 or 8
    int quad_ctas_per_sm = 8;  // persistent fit/decode grid = SMs * this (capped by the work)
    int quad_split = 32;       // candidates with a bbox side above this (px) take a CTA each; 0: none
    int band_cap = 2048;       // runs of a band unioned in shared memory (256..2048); more: fallback
    int fit_merged = 0;        // 1: big and small candidates in one fit-and-decode launch
    int persistent = 0;        // 1: the whole batch as one persistent launch (k_persistent.cu)
    int persist_ctas = 0;      // CTAs of that launch (0: every SM's resident maximum)
};

// A second stream and two events for the parallel branch of the pipeline
// (the CTA path of big candidates); events without timing.
struct ForkJoin {
    void* stream;
    void* fork_event;
    void* join_event;
};

// Fills the stats fields of a host BatchDesc for `rows` tile rows per CTA.
inline void set_stats_rows(BatchDesc& d, int rows) {
    d.stats_rows = rows;
    int run = 0;
    for (int f = 0; f < d.frames; ++f) {
        d.stats_prefix[f] = run;
        run += (d.f[f].tile_h + rows - 1) / rows;
    }
    d.stats_prefix[d.frames] = run;
    d.stats_ctas = run;
}

BDGB_HD inline bd_detection* result_detections(FrameResultHeader* h) {
    return reinterpret_cast<bd_detection*>(h + 1);
}

BDGB_HD inline size_t result_bytes(int max_detections) {
    return sizeof(FrameResultHeader) + 2 * static_cast<size_t>(max_detections) * sizeof(bd_detection);
}

// Launch sequence of one batch on one stream (k_finalize.cu).  `io` is a
// device array of FrameIO, one per frame.  With `fork` the big-candidate
// kernel runs on fork->stream beside the warp-per-candidate kernel.  When
// stage_events is not null (no fork then) it holds kStageCount + 1
// cudaEvent_t, recorded before the first kernel and after every kernel, so
// consecutive events bracket one stage.
constexpr int kStageCount = 8;
// The persistent launch: how long a CTA waits for a queue slot before the
// launch gives up (the status then says so), and a test hook that withholds
// one item of frame `stall_frame` (-1: none) so that the wait runs out.
struct PersistParams {
    uint64_t timeout_ns = 1000000000ull;
    int stall_frame = -1;
};
// Per-device kernel attributes; call with the device current before the
// first enqueue.  0 on success.
int prepare_pipeline();
extern const char* const kStageNames[kStageCount];
void enqueue_pipeline(const BatchDesc* device_desc, const BatchDesc& host_desc,
                      const FrameIO* device_io, void* stream, const LaunchConfig& launch,
                      int sm_count, const ForkJoin* fork, void* const* stage_events = nullptr);

// The persistent launch of a batch (k_persistent.cu): one kernel whose CTAs
// pull (frame, stage, unit) items from `queue` until every frame is done.
int prepare_persistent();
void enqueue_persistent(const BatchDesc* device_desc, const BatchDesc& host_desc,
                        const FrameIO* device_io, WorkQueue* queue, void* stream,
                        const LaunchConfig& launch, int sm_count, const PersistParams& persist);

}  // namespace bdgb
