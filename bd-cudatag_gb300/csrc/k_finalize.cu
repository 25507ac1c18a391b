// Stage 7 (de-duplication, sort, records) and the launch sequence of a
// batch: prepare_pipeline, stage names, enqueue_pipeline.

#include <atomic>

#include "stage_finalize.cuh"

namespace bdgb {

__global__ void __launch_bounds__(kFinalThreads) k_finalize(const BatchDesc* __restrict__ b) {
    __shared__ FinalSmem sm;
    stage_finalize(b, blockIdx.x >> 1, blockIdx.x & 1, sm);
}


// Resident CTAs per SM of k_fit_decode_all (its grid fills the GPU once).
std::atomic<int> g_fit_all_ctas_per_sm{1};

int prepare_pipeline() {
    // Shared memory beyond 48 KB per block needs an opt-in, per device.
    if (cudaFuncSetAttribute(k_binarize_runs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(band_smem_bytes(kMaxBandCap, BD_MAX_WIDTH / 32))) !=
        cudaSuccess) {
        return -1;
    }
    if (cudaFuncSetAttribute(k_fit_decode_all, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(fit_all_smem_bytes())) != cudaSuccess) {
        return -1;
    }
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fit_decode_all, 256, fit_all_smem_bytes()) ==
        cudaSuccess) {
        g_fit_all_ctas_per_sm.store(std::max(1, per_sm));
    }
    return cudaFuncSetAttribute(k_fit_decode, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(kMaxQuadWarps * quad_smem_per_warp())) == cudaSuccess
               ? 0
               : -1;
}

const char* const kStageNames[kStageCount] = {
    "stats", "binarize_runs", "merge", "region_stats", "cand_count",
    "fit_decode_big", "fit_decode", "finalize"};

void enqueue_pipeline(const BatchDesc* dd, const BatchDesc& hd, const FrameIO* io, void* stream_ptr,
                      const LaunchConfig& lc, int sm_count, const ForkJoin* fork,
                      void* const* stage_events) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);
    auto mark = [&](int k) {
        if (stage_events) cudaEventRecord(static_cast<cudaEvent_t>(stage_events[k]), s);
    };
    const int bands = hd.total_bands;
    int items = 0;  // candidate-family pairs at the caps
    for (int f = 0; f < hd.frames; ++f) {
        items += hd.f[f].max_candidates * __builtin_popcount(hd.f[f].families & 3u);
    }
    const int warps = lc.quad_warps;
    const int quad_grid =
        std::max(1, std::min((items + warps - 1) / warps, sm_count * lc.quad_ctas_per_sm));
    mark(0);
    k_stats<<<hd.stats_ctas, 256, 0, s>>>(dd, io);
    mark(1);
    int words_max = 1;
    for (int f = 0; f < hd.frames; ++f) words_max = std::max(words_max, hd.f[f].words);
    k_binarize_runs<<<bands, 256, band_smem_bytes(lc.band_cap, words_max), s>>>(dd, io, lc.band_cap,
                                                                                 words_max);
    mark(2);
    int row_cap_max = 1;
    for (int f = 0; f < hd.frames; ++f) row_cap_max = std::max(row_cap_max, hd.f[f].row_cap);
    k_merge<<<bands, 256, 2 * row_cap_max * sizeof(uint32_t), s>>>(dd, io, row_cap_max);
    mark(3);
    k_region_stats<<<bands, 256, 0, s>>>(dd, io);
    mark(4);
    const int split = lc.quad_split;
    int th_max = 1;
    for (int f = 0; f < hd.frames; ++f) th_max = std::max(th_max, hd.f[f].tile_h);
    k_cand_count<<<bands, 256, (th_max + 1) * sizeof(uint32_t), s>>>(dd, io, split);
    mark(5);
    int cands = 0;
    for (int f = 0; f < hd.frames; ++f) cands += hd.f[f].max_candidates;
    const int big_grid = std::max(1, std::min(cands, sm_count));
    const size_t quad_smem = warps * quad_smem_per_warp();
    if (lc.fit_merged) {
        // One launch for both paths: the big candidates' CTA time is part of
        // the fit_decode stage, and the fit_decode_big stage stays empty.
        mark(6);
        k_fit_decode_all<<<sm_count * g_fit_all_ctas_per_sm.load(), 256, fit_all_smem_bytes(), s>>>(dd, io);
        mark(7);
    } else if (split > 0 && fork && !stage_events) {
        // Big candidates on a parallel branch (a fork/join in the graph).
        cudaStream_t s2 = static_cast<cudaStream_t>(fork->stream);
        cudaEventRecord(static_cast<cudaEvent_t>(fork->fork_event), s);
        cudaStreamWaitEvent(s2, static_cast<cudaEvent_t>(fork->fork_event), 0);
        k_fit_decode_big<<<big_grid, 256, 0, s2>>>(dd, io, split);
        cudaEventRecord(static_cast<cudaEvent_t>(fork->join_event), s2);
        k_fit_decode<<<quad_grid, warps * 32, quad_smem, s>>>(dd, io);
        cudaStreamWaitEvent(s, static_cast<cudaEvent_t>(fork->join_event), 0);
        mark(6);
        mark(7);
    } else {
        if (split > 0) k_fit_decode_big<<<big_grid, 256, 0, s>>>(dd, io, split);
        mark(6);
        k_fit_decode<<<quad_grid, warps * 32, quad_smem, s>>>(dd, io);
        mark(7);
    }
    k_finalize<<<hd.frames * 2, kFinalThreads, 0, s>>>(dd);
    mark(8);
}

}  // namespace bdgb
