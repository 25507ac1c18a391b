// Tile statistics of one frame without any allocation.
//
// Some callers cannot allocate device memory at the time they want to run
// detection work: a camera or ISP callback that must not block, a host that
// hands this library a fixed memory budget up front (real-time or
// safety-certified systems forbid allocation after start-up), or code that
// runs inside someone else's allocator and stream discipline.  For them,
// bd_tile_stats_device_noalloc computes the first pipeline stage (per-tile
// min/max and the frame's noise-floor and Otsu references, the same values
// k_stats produces inside a detector) using only the caller's input and
// output buffers plus one small scratch array that is part of the library
// image itself: g_noalloc_scratch below, a file-scope __device__ array that
// every GPU which loads the library holds until the process exits.
//
// The scratch is shared by every call on a device and keeps the last call's
// contents; each call clears what must start at zero.  Calls whose GPU work
// overlaps (two streams, or two host threads) race on it and give wrong
// results: serialise them.

#include <cuda_runtime.h>

#include <climits>
#include <cstdint>

#include "bdcudatag/bdcudatag.h"
#include "bdcudatag/bdcudatag_gb300.h"
#include "kernels_common.cuh"
#include "pipeline.cuh"

namespace bdgb {

void set_last_error(const char* message);  // capi.cpp

namespace {

struct NoAllocScratch {
    uint32_t span_hist[256];
    uint32_t mean_hist[64];
    uint32_t top_enc;      // tile_h - first contrasting tile row (0: none)
    uint32_t bottom_enc;   // last contrasting tile row + 1 (0: none)
    uint32_t done;         // CTAs finished
};

// 2 KiB, independent of the frame size.
constexpr size_t kNoAllocScratchBytes = 2048;
static_assert(sizeof(NoAllocScratch) <= kNoAllocScratchBytes, "scratch too small");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The per-frame part of k_stats (k_front.cu) with explicit buffers, built
// from the same device routines (tile_pair_stats, frame_references,
// roi_tile_rows): one CTA per tile row, one thread per tile pair; the last
// CTA turns the histograms into the frame references.
__global__ void __launch_bounds__(256) k_tile_stats_noalloc(const uint8_t* __restrict__ gray,
                                                            int W, int H, int64_t stride,
                                                            uint8_t* __restrict__ tile_min,
                                                            uint8_t* __restrict__ tile_max,
                                                            NoAllocScratch* __restrict__ sc,
                                                            uint32_t* __restrict__ frame_out) {
    __shared__ uint32_t s_span[256];
    __shared__ uint32_t s_mean[64];
    __shared__ int s_lo, s_hi, s_last;
    __shared__ RefSmem s_ref;

    const int tid = threadIdx.x;
    const int ty = blockIdx.x;
    const int tw = (W + kTile - 1) / kTile;
    const int th = (H + kTile - 1) / kTile;
    s_span[tid] = 0;
    if (tid < 64) s_mean[tid] = 0;
    if (tid == 0) {
        s_lo = INT_MAX;
        s_hi = -1;
    }
    __syncthreads();

    const bool vec16 = ((reinterpret_cast<uintptr_t>(gray) | static_cast<uintptr_t>(stride)) & 15u) == 0;
    const int pairs = (tw + 1) >> 1;
    int lo = INT_MAX, hi = -1;
    for (int pair = tid; pair < pairs; pair += blockDim.x) {
        TileStat t[2];
        tile_pair_stats(gray, stride, W, H, ty, pair, vec16, &t[0], &t[1]);
        for (int k = 0; k < 2; ++k) {
            if (t[k].mn > 255u) continue;  // no second tile in this pair
            const int tx = 2 * pair + k;
            tile_min[ty * tw + tx] = static_cast<uint8_t>(t[k].mn);
            tile_max[ty * tw + tx] = static_cast<uint8_t>(t[k].mx);
            atomicAdd(&s_span[(t[k].mx - t[k].mn) & 0xffu], 1u);
            atomicAdd(&s_mean[t[k].mean >> 2], 1u);
            if (static_cast<int>(t[k].mx - t[k].mn) >= kMinTileContrast) {
                lo = min(lo, tx);
                hi = max(hi, tx);
            }
        }
    }
    if (hi >= 0) {
        atomicMin(&s_lo, lo);
        atomicMax(&s_hi, hi);
    }
    __syncthreads();
    if (tid == 0 && s_hi >= 0) {
        atomicMax(&sc->top_enc, static_cast<uint32_t>(th - ty));
        atomicMax(&sc->bottom_enc, static_cast<uint32_t>(ty + 1));
    }
    if (s_span[tid]) atomicAdd(&sc->span_hist[tid], s_span[tid]);
    if (tid < 64 && s_mean[tid]) atomicAdd(&sc->mean_hist[tid], s_mean[tid]);
    __threadfence();
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(&sc->done, 1u) == static_cast<uint32_t>(th - 1);
    __syncthreads();
    if (!s_last) return;
    __threadfence();

    frame_references(sc->span_hist, sc->mean_hist, s_ref, &frame_out[0], &frame_out[1]);
    if (tid == 0) frame_out[2] = roi_tile_rows(__ldcg(&sc->top_enc), __ldcg(&sc->bottom_enc), th);
}

// Device address of g_noalloc_scratch on the current device.  Looked up on
// every call (the lookup allocates nothing), so it stays right after a
// device reset or under another context.
int32_t scratch_address(void** out) {
    void* ptr = nullptr;
    const cudaError_t st = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (st != cudaSuccess || !ptr) {
        set_last_error("bd_tile_stats_device_noalloc: cudaGetSymbolAddress failed for the "
                       "scratch array");
        return BD_ERROR_CUDA;
    }
    *out = ptr;
    return BD_OK;
}

}  // namespace
}  // namespace bdgb

extern "C" int32_t bd_tile_stats_device_noalloc(const uint8_t* gray_device, int32_t width,
                                                int32_t height, int32_t stride,
                                                uint8_t* tile_min_device, uint8_t* tile_max_device,
                                                uint32_t* frame_device, void* cuda_stream) {
    using namespace bdgb;
    if (!gray_device || !tile_min_device || !tile_max_device || !frame_device) {
        set_last_error("bd_tile_stats_device_noalloc: null buffer pointer");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (width < 16 || width > BD_NOALLOC_MAX_WIDTH || height < 16 || height > BD_NOALLOC_MAX_HEIGHT) {
        set_last_error("bd_tile_stats_device_noalloc: frame size out of range "
                       "(16..8192 x 16..16384)");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    if (stride < width) {
        set_last_error("stride is smaller than the image width");
        return BD_ERROR_INVALID_ARGUMENT;
    }
    void* scratch = nullptr;
    const int32_t rc = scratch_address(&scratch);
    if (rc != BD_OK) return rc;
    cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
    // Both calls return their own status, so an error left pending by
    // earlier, unrelated work is neither reported here nor cleared.
    cudaError_t st = cudaMemsetAsync(scratch, 0, sizeof(NoAllocScratch), s);
    if (st == cudaSuccess) {
        const int tile_h = (height + kTile - 1) / kTile;
        const uint8_t* g = gray_device;
        int w = width, h = height;
        int64_t stride64 = stride;
        NoAllocScratch* sc = static_cast<NoAllocScratch*>(scratch);
        void* args[] = {&g, &w, &h, &stride64, &tile_min_device, &tile_max_device, &sc, &frame_device};
        st = cudaLaunchKernel(reinterpret_cast<const void*>(k_tile_stats_noalloc), dim3(tile_h), dim3(256),
                              args, 0, s);
    }
    if (st != cudaSuccess) {
        set_last_error(cudaGetErrorString(st));
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}
