// CPU ORACLE -- test infrastructure, not part of the product.
//
// A sequential C++ restatement of the reference bdcudatag per-frame pipeline
// (reference detector/src/gpu_detector.cu:104-1601 plus the host homography
// :1739-1774 and the result handling :2100-2127).  Only tests/, the smoke
// check in __graft_entry__.py and bench.py's CPU-baseline leg may load it.
//
// Parity pin: the oracle reproduces the reference's own known-answer tests
// (detector/tests/test_detector.cpp) and, on the reference's own benchmark
// scenes (built from detector/bench/scenes.hpp by oracle/build_ref.sh and
// hashed into tests/golden/), the reference's published recall, wrong-id and
// corner-error figures.  The reference GPU library cannot run in the build
// container (no GPU) or on the Arm GPU host (no aarch64 cross compiler to
// carry it there), so no stage of it is compared bit for bit.
//
// Two deliberate conventions, shared with the CUDA pipeline:
//  * Canonical order where the reference uses atomics: candidates inside an
//    area bin are ordered by root slot id, and decoded detections take slots
//    in candidate order.  The reference's order there is whatever its atomic
//    counters produce (gpu_detector.cu:632, :1525); the detection set is the
//    same whenever the candidate and detection caps are not exceeded.
//  * Floating point: every FP32 expression is evaluated in source order with
//    one rounding per operation (built with -ffp-contract=off), and the four
//    transcendental calls use bd-cudatag_gb300/csrc/detmath.h.  The reference
//    build lets nvcc fuse multiply-adds and uses CUDA's libm, so its corners
//    and margins can differ from ours in the last bits.
#pragma once

#include <stdint.h>

#include "bdcudatag/bdcudatag.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bdo_frame bdo_frame;

// Runs the full pipeline on one frame.  config may be NULL (defaults).
// Returns NULL on invalid arguments.
bdo_frame* bdo_run(const uint8_t* gray, int32_t width, int32_t height, int32_t stride,
                   int32_t family, const bd_config* config);
void bdo_free(bdo_frame* frame);

// Final detections as bd_detector_detect_host would return them: writes
// min(found, capacity) records (homography filled) and returns `found`.
int32_t bdo_detections(const bdo_frame* frame, bd_detection* out, int32_t capacity);

// counts[0..4]: candidates (uncapped), detections, runs, quads, ROI tile rows.
void bdo_counts(const bdo_frame* frame, uint32_t counts[5]);

// Resolved geometry: [tile_w, tile_h, words, row_cap, max_candidates,
// max_detections, dim, max_hamming, candidate_count]
void bdo_geometry(const bdo_frame* frame, int32_t out[9]);

// Copies a named stage buffer into dst (at most dst_bytes).  Returns the
// buffer's full size in bytes, or -1 for an unknown name.  Names:
//  tile_min tile_max tile_mean thresh active (u8[T]); span_hist (u32[256]);
//  mean_hist (u32[64]); ref (u32[2]); row_active (u8[tile_h]);
//  row_start row_end (i32[tile_h]); bits (u32[H*words]); row_count (u32[H]);
//  runs (u32[slots]); label (u32[slots], root slot, 0xffffffff if unused);
//  area (u32[slots]); bbox (u32[4*slots]) -- both valid at root slots only;
//  candidates (u32[n]); hull_quads quads (f32[max_candidates*8], NaN when
//  no quad); decodes (i32+i32+f32+8*f32 per candidate: id, hamming, margin,
//  corners; id -1 when nothing decoded).
int64_t bdo_stage(const bdo_frame* frame, const char* name, void* dst, int64_t dst_bytes);

// Detects every frame of a set on `threads` host threads, one (frame,
// family) pair per task, one family per family bit.  out holds frames*2 blocks of max_detections
// records; counts[frame*2+family] = found (or -1 if that family was not
// requested).  Returns 0 on success.
int32_t bdo_detect_many(int32_t frames, const uint8_t* const* grays, const int32_t* widths,
                        const int32_t* heights, const int32_t* strides,
                        const uint32_t* family_masks, const bd_config* config,
                        int32_t threads, bd_detection* out, int32_t max_detections,
                        int32_t* counts);

// FP64 re-fit: the hull, quad and edge-refinement steps of every candidate
// evaluated in double precision (C library sin/cos/atan2/hypot), from the
// frame's integer stages.  `gray` must be the image the frame was run on.
// hull_out and quads_out hold candidate_count * 8 doubles (NaN when the
// candidate gives no quad).  Returns candidate_count.
int32_t bdo_refit64(const bdo_frame* frame, const uint8_t* gray, double* hull_out,
                    double* quads_out);

// The host homography of the result records (reference fill_homography,
// gpu_detector.cu:1739-1774) from FP64 corners, kept in FP64.
void bdo_homography64(const double corners[8], double H[9]);

// The deterministic math helpers, exported for the accuracy test.
float bdo_sinf(float x);
float bdo_cosf(float x);
float bdo_atan2f(float y, float x);

#ifdef __cplusplus
}
#endif
