// Stage 7 (de-duplication, sort, records) and the launch sequence of a
// batch: prepare_pipeline, stage names, enqueue_pipeline.

#include "kernels_common.cuh"
#include "kernels.cuh"

namespace bdgb {

// ===========================================================================
// 9. Finalize one (frame, family): detections in candidate order (first
//    max_detections), de-duplication, stable sort by id, homography
//    (reference k_finalize :1542-1601, host fill_homography :1739-1774 --
//    FP64 here as there).
// ===========================================================================

__global__ void __launch_bounds__(kFinalThreads) k_finalize(const BatchDesc* __restrict__ b) {
    __shared__ DecodeOut s_in[kMaxDetectionsCap];
    __shared__ DecodeOut s_out[kMaxDetectionsCap];
    __shared__ int s_in_src[kMaxDetectionsCap], s_out_src[kMaxDetectionsCap];  // candidate index
    __shared__ float s_cx[kMaxDetectionsCap], s_cy[kMaxDetectionsCap];
    __shared__ uint32_t s_warp[kFinalThreads / 32];
    __shared__ int s_count, s_kept;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int fi = blockIdx.x >> 1;
    const int fam = blockIdx.x & 1;
    const FrameDesc& d = b->f[fi];
    const FrameState* st = d.state;
    FrameResultHeader* hdr = d.result;
    if (fam == 0 && tid < 5) hdr->counts[tid] = st->counts[tid];
    if (fam == 0 && tid == 5) hdr->pad = 0;
    if (!(d.families & (1u << fam))) {
        if (tid == 0) hdr->found[fam] = 0;
        return;
    }
    const int n = static_cast<int>(st->n_candidates);
    const int maxd = d.max_detections;
    const DecodeOut* dec = d.decodes + static_cast<int64_t>(fam) * d.max_candidates;
    if (tid == 0) s_count = 0;
    __syncthreads();
    // Ordered compaction of the decoded candidates.
    for (int c = 0; c < n; c += kFinalThreads) {
        const int i = c + tid;
        const bool ok = i < n && dec[i].id >= 0;
        const unsigned bal = __ballot_sync(kFull, ok);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        int before = s_count;
        for (int w2 = 0; w2 < warp; ++w2) before += static_cast<int>(s_warp[w2]);
        const int pos = before + __popc(bal & lanemask_lt());
        if (ok && pos < maxd) {
            s_in[pos] = dec[i];
            s_in_src[pos] = i;
        }
        __syncthreads();
        if (tid == 0) {
            int add = 0;
            for (int w2 = 0; w2 < kFinalThreads / 32; ++w2) add += static_cast<int>(s_warp[w2]);
            s_count = s_count + add;
        }
        __syncthreads();
        if (s_count >= maxd) break;
    }
    const int m = min(s_count, maxd);
    // De-duplication in arrival order, one warp.
    if (warp == 0) {
        int kept = 0;
        for (int i = 0; i < m; ++i) {
            const DecodeOut& dd = s_in[i];
            float side = 0.0f, cx = 0.0f, cy = 0.0f;
            for (int k = 0; k < 4; ++k) {
                const int j = (k + 1) & 3;
                side += bdmath::hypot(dd.corners[j * 2] - dd.corners[k * 2],
                                      dd.corners[j * 2 + 1] - dd.corners[k * 2 + 1]);
                cx += dd.corners[k * 2];
                cy += dd.corners[k * 2 + 1];
            }
            side *= 0.25f;
            cx *= 0.25f;
            cy *= 0.25f;
            const float limit = 0.35f * side;
            int duplicate = -1;
            for (int k0 = 0; k0 < kept && duplicate < 0; k0 += 32) {
                const int k = k0 + lane;
                const bool hit = k < kept && s_out[k].id == dd.id && fabsf(s_cx[k] - cx) < limit &&
                                 fabsf(s_cy[k] - cy) < limit;
                const unsigned bal = __ballot_sync(kFull, hit);
                if (bal) duplicate = k0 + __ffs(bal) - 1;
            }
            __syncwarp();
            if (lane == 0) {
                if (duplicate >= 0) {
                    if (dd.margin > s_out[duplicate].margin) {
                        s_out[duplicate] = dd;
                        s_out_src[duplicate] = s_in_src[i];
                        s_cx[duplicate] = cx;
                        s_cy[duplicate] = cy;
                    }
                } else if (kept < maxd) {
                    s_out[kept] = dd;
                    s_out_src[kept] = s_in_src[i];
                    s_cx[kept] = cx;
                    s_cy[kept] = cy;
                }
            }
            if (duplicate < 0 && kept < maxd) ++kept;
            __syncwarp();
        }
        if (lane == 0) s_kept = kept;
    }
    __syncthreads();
    const int kept = s_kept;
    bd_detection* dets = result_detections(hdr) + static_cast<int64_t>(fam) * maxd;
    for (int i = tid; i < kept; i += kFinalThreads) {
        const int id = s_out[i].id;
        int rank = 0;
        for (int j = 0; j < kept; ++j) {
            const int oj = s_out[j].id;
            rank += (oj < id || (oj == id && j < i)) ? 1 : 0;
        }
        bd_detection r;
        r.id = id;
        r.hamming = s_out[i].hamming;
        r.decision_margin = s_out[i].margin;
        for (int k = 0; k < 8; ++k) r.corners[k] = s_out[i].corners[k];
        r.reserved = 0;
        const float* hsrc = d.dec_h + (static_cast<int64_t>(fam) * d.max_candidates + s_out_src[i]) * 9;
        for (int k = 0; k < 9; ++k) r.homography[k] = hsrc[k];
        dets[rank] = r;
    }
    if (tid == 0) hdr->found[fam] = static_cast<uint32_t>(kept);
}


int prepare_pipeline() {
    // Shared memory beyond 48 KB per block needs an opt-in, per device.
    if (cudaFuncSetAttribute(k_binarize_runs, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             static_cast<int>(band_smem_bytes(kMaxBandCap, BD_MAX_WIDTH / 32))) !=
        cudaSuccess) {
        return -1;
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
    if (split > 0 && fork && !stage_events) {
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
