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

size_t quad_smem_per_warp() { return sizeof(QuadSmem); }

}  // namespace bdgb
