// Kernels of the batched pipeline (one launch per stage for a whole batch)
// and the launch-shape constants they share with the launch sequence.  Stage
// map, with the reference kernels each one replaces
// (detector/src/gpu_detector.cu):
//   k_stats          tile min/max/mean, span+mean histograms, active extents,
//                    and (last CTA of a frame) noise floor + Otsu + ROI rows
//                    <- k_tile_stats :104, k_tile_histograms :140,
//                       k_tile_reference :174, k_build_row_roi :282
//   k_binarize_runs  3x3 pooled threshold, bit-packed binarization of the
//                    row band, run extraction, band-local components
//                    <- k_tile_threshold :237, k_binarize :362,
//                       k_find_runs :427, k_merge_runs :509 (inside a band)
//   k_merge          unions across band boundaries  <- k_merge_runs :509
//   k_region_stats   area / bbox per root  <- k_region_stats :562
//   k_cand_count     root flattening, tag-like filter, ordered per-band
//                    bin ranks; the frame's last CTA computes the bin bases
//                    and places the candidates  <- k_collect_candidates :591,
//                    k_order_candidates :642
//   k_fit_decode     warp per (candidate, family): hull, four corners, edge
//   k_fit_decode_big refinement and decode (CTA per big candidate)
//                    <- k_fit_quads :1081, k_decode_quads :1438
//   k_finalize       de-duplication, sort by id, records
//                    <- k_finalize :1542, host fill_homography :1739
// Files: k_front.cu (stats .. cand_count), k_quad.cu (fit/decode),
// k_finalize.cu (finalize and the launch sequence).
#pragma once

#include <cstddef>
#include <cstdint>

#include "pipeline.cuh"

namespace bdgb {

constexpr int kMaxBandCap = 2048;
// Dynamic shared memory of k_binarize_runs: six arrays of `cap` run
// entries, the band's bit rows (kTile rows of `words` words), then the row
// (byte) of each run entry.
__host__ __device__ constexpr size_t band_smem_bytes(int cap, int words) {
    return (6 * static_cast<size_t>(cap) + kTile * static_cast<size_t>(words)) * sizeof(uint32_t) +
           static_cast<size_t>(cap);
}

constexpr int kFinalThreads = 256;

__global__ void k_stats(const BatchDesc* b, const FrameIO* io);
__global__ void k_binarize_runs(const BatchDesc* b, const FrameIO* io, int cap, int bits_words);
__global__ void k_merge(const BatchDesc* b, const FrameIO* io, int row_cap_max);
__global__ void k_region_stats(const BatchDesc* b, const FrameIO* io);
__global__ void k_cand_count(const BatchDesc* b, const FrameIO* io, int split_px);
__global__ void k_fit_decode(const BatchDesc* b, const FrameIO* io);
__global__ void k_fit_decode_big(const BatchDesc* b, const FrameIO* io, int split_px);
__global__ void k_fit_decode_all(const BatchDesc* b, const FrameIO* io);
__global__ void k_finalize(const BatchDesc* b);

// Dynamic shared memory of one k_fit_decode warp, and of a k_fit_decode_all
// CTA (256 threads).
size_t quad_smem_per_warp();
size_t fit_all_smem_bytes();

}  // namespace bdgb
