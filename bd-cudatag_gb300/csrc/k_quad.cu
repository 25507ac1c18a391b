// Quad fit and decode as one launch per stage for a whole batch:
// k_fit_decode (one warp per small (candidate, family) item) and
// k_fit_decode_big (one CTA per big candidate), over the work lists that
// k_cand_count writes (stage_quad.cuh holds the device functions).

#include "stage_quad.cuh"

namespace bdgb {

// Flattened work list of (frame, candidate, family) items over the
// candidates at or below the big-candidate split (the back of
// FrameDesc::fit_list), the families of a candidate adjacent; warp w of CTA
// c takes items c * warps + w, then strides by grid * warps.  Each warp builds the candidate's hull itself (the
// warp of the frame's lowest family also stores it), so the families of a
// candidate proceed concurrently and warps never wait for one another after
// the work-list prefix.
__global__ void __launch_bounds__(256) k_fit_decode(const BatchDesc* __restrict__ b,
                                                    const FrameIO* __restrict__ io) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ int s_prefix[kMaxFrames + 1];
    __shared__ float s_uv[2][8];
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const int warps = blockDim.x >> 5;
    if (tid < 16) {
        const int fam = tid >> 3, c = tid & 7;
        s_uv[fam][c] = (c + 0.5f) / static_cast<float>(family_dim(fam));
    }
    if (tid == 0) {
        int run = 0;
        for (int f = 0; f < b->frames; ++f) {
            s_prefix[f] = run;
            run += static_cast<int>(b->f[f].state->n_small) * __popc(b->f[f].families & 3u);
        }
        s_prefix[b->frames] = run;
    }
    __syncthreads();
    QuadSmem& sm = reinterpret_cast<QuadSmem*>(s_dyn)[warp];
    const int total = s_prefix[b->frames];
    // Probe direction of this lane (reference :1134-1170).
    float ux, uy;
    {
        const float angle =
            6.28318530718f * static_cast<float>(lane) / static_cast<float>(kFitDirections);
        bdmath::sincos(angle, &uy, &ux);
    }

    for (int item = blockIdx.x * warps + warp; item < total; item += gridDim.x * warps) {
        int fi = 0;
        while (s_prefix[fi + 1] <= item) ++fi;
        const int nfam = __popc(b->f[fi].families & 3u);
        const int local = item - s_prefix[fi];
        const int k = local / nfam;
        fit_small_item(b, io, fi, k, local - k * nfam, ux, uy, s_uv, sm, lane);
    }
}

__global__ void __launch_bounds__(256, 3) k_fit_decode_big(const BatchDesc* __restrict__ b,
                                                        const FrameIO* __restrict__ io, int split_px) {
    __shared__ BigSmem sm;
    __shared__ int s_prefix[kMaxFrames + 1];
    __shared__ float s_uv[2][8];
    const int tid = threadIdx.x;
    const int lane = tid & 31;
    if (tid < 16) {
        const int fam = tid >> 3, c = tid & 7;
        s_uv[fam][c] = (c + 0.5f) / static_cast<float>(family_dim(fam));
    }
    if (tid == 0) {
        int run = 0;
        for (int f = 0; f < b->frames; ++f) {
            s_prefix[f] = run;
            run += static_cast<int>(b->f[f].state->n_big);
        }
        s_prefix[b->frames] = run;
    }
    __syncthreads();
    const int total = s_prefix[b->frames];
    float ux, uy;
    {
        const float angle =
            6.28318530718f * static_cast<float>(lane) / static_cast<float>(kFitDirections);
        bdmath::sincos(angle, &uy, &ux);
    }
    // Big candidate k of the batch (frames in order, each frame's list as
    // k_cand_count wrote it) goes to CTA k % grid.
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        int fi = 0;
        while (s_prefix[fi + 1] <= item) ++fi;
        fit_big_item(b, io, fi, item - s_prefix[fi], ux, uy, s_uv, sm);
    }
}

// Both fit-and-decode paths in one launch of 8-warp CTAs: a CTA first takes
// big candidates of the batch one at a time (fit_big_item), then its warps
// take (small candidate, family) pairs one at a time (fit_small_item), both
// handed out by counters in frame 0's state.  No fork in the graph, so a
// batch uses one hardware queue.
__global__ void __launch_bounds__(256, 3) k_fit_decode_all(const BatchDesc* __restrict__ b,
                                                        const FrameIO* __restrict__ io) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ int s_big[kMaxFrames + 1];
    __shared__ int s_small[kMaxFrames + 1];
    __shared__ float s_uv[2][8];
    __shared__ uint32_t s_item;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid < 16) {
        const int fam = tid >> 3, c = tid & 7;
        s_uv[fam][c] = (c + 0.5f) / static_cast<float>(family_dim(fam));
    }
    if (tid == 0) {
        int big = 0, small = 0;
        for (int f = 0; f < b->frames; ++f) {
            s_big[f] = big;
            s_small[f] = small;
            big += static_cast<int>(b->f[f].state->n_big);
            small += static_cast<int>(b->f[f].state->n_small) * __popc(b->f[f].families & 3u);
        }
        s_big[b->frames] = big;
        s_small[b->frames] = small;
    }
    __syncthreads();
    float ux, uy;
    {
        const float angle =
            6.28318530718f * static_cast<float>(lane) / static_cast<float>(kFitDirections);
        bdmath::sincos(angle, &uy, &ux);
    }
    FrameState* counters = b->f[0].state;
    const uint32_t total_big = static_cast<uint32_t>(s_big[b->frames]);
    for (;;) {
        if (tid == 0) s_item = atomicAdd(&counters->batch_big_next, 1u);
        __syncthreads();
        const uint32_t item = s_item;
        if (item >= total_big) break;
        int fi = 0;
        while (s_big[fi + 1] <= static_cast<int>(item)) ++fi;
        fit_big_item(b, io, fi, static_cast<int>(item) - s_big[fi], ux, uy, s_uv,
                     *reinterpret_cast<BigSmem*>(s_dyn));
    }
    __syncthreads();  // the big path's shared memory becomes the warps' own
    QuadSmem& sm = reinterpret_cast<QuadSmem*>(s_dyn)[warp];
    const uint32_t total_small = static_cast<uint32_t>(s_small[b->frames]);
    for (;;) {
        uint32_t item = 0;
        if (lane == 0) item = atomicAdd(&counters->batch_small_next, 1u);
        item = __shfl_sync(kFull, item, 0);
        if (item >= total_small) break;
        int fi = 0;
        while (s_small[fi + 1] <= static_cast<int>(item)) ++fi;
        const int nfam = __popc(b->f[fi].families & 3u);
        const int local = static_cast<int>(item) - s_small[fi];
        const int k = local / nfam;
        fit_small_item(b, io, fi, k, local - k * nfam, ux, uy, s_uv, sm, lane);
    }
}

size_t quad_smem_per_warp() { return sizeof(QuadSmem); }

size_t fit_all_smem_bytes() { return std::max(sizeof(BigSmem), 8 * sizeof(QuadSmem)); }

}  // namespace bdgb
