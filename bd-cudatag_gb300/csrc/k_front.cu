// Stages 1-5 of the batched pipeline as one launch per stage for a whole
// batch: each kernel finds its frame and unit from blockIdx and runs the
// stage's device function (stage_front.cuh).

#include "stage_front.cuh"

namespace bdgb {

__global__ void __launch_bounds__(256) k_stats(const BatchDesc* __restrict__ b,
                                               const FrameIO* __restrict__ io) {
    __shared__ StatsSmem sm;
    int fi = 0;
    {
        int lo = 0, hi = b->frames - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (b->stats_prefix[mid] <= static_cast<int>(blockIdx.x)) lo = mid; else hi = mid - 1;
        }
        fi = lo;
    }
    if (!io[fi].gray) return;  // slot not used in this launch
    stage_stats(b, io, fi, blockIdx.x - b->stats_prefix[fi], sm);
}

__global__ void __launch_bounds__(256, 6) k_binarize_runs(const BatchDesc* __restrict__ b,
                                                       const FrameIO* __restrict__ io, int cap,
                                                       int bits_words) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ BinSmem sm;
    const int fi = frame_of_band(b, blockIdx.x);
    if (!io[fi].gray) return;
    stage_binarize(b, io, fi, blockIdx.x - b->band_prefix[fi], cap, bits_words, sm, s_dyn);
}

__global__ void __launch_bounds__(256, 2) k_merge(const BatchDesc* __restrict__ b,
                                               const FrameIO* __restrict__ io, int row_cap_max) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    const int fi = frame_of_band(b, blockIdx.x);
    if (!io[fi].gray) return;
    stage_merge(b, fi, blockIdx.x - b->band_prefix[fi], row_cap_max, s_dyn);
}

__global__ void __launch_bounds__(256) k_region_stats(const BatchDesc* __restrict__ b,
                                                      const FrameIO* __restrict__ io) {
    const int fi = frame_of_band(b, blockIdx.x);
    if (!io[fi].gray) return;
    stage_region(b, fi, blockIdx.x - b->band_prefix[fi]);
}

__global__ void __launch_bounds__(256) k_cand_count(const BatchDesc* __restrict__ b,
                                                    const FrameIO* __restrict__ io, int split_px) {
    // Candidates before each band of the frame (tallest frame's bands + 1,
    // sized at launch).
    extern __shared__ uint32_t s_cprefix[];
    __shared__ CandSmem sm;
    const int fi = frame_of_band(b, blockIdx.x);
    if (!io[fi].gray) return;
    stage_cand(b, fi, blockIdx.x - b->band_prefix[fi], split_px, sm, s_cprefix);
}

}  // namespace bdgb
