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
#include <mutex>

#include "bdcudatag/bdcudatag.h"
#include "bdcudatag/bdcudatag_gb300.h"
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

constexpr unsigned kFull = 0xffffffffu;

// The per-frame part of k_stats (k_front.cu) with explicit buffers: one CTA
// per tile row; the last CTA turns the histograms into the frame references.
__global__ void __launch_bounds__(256) k_tile_stats_noalloc(const uint8_t* __restrict__ gray,
                                                            int W, int H, int64_t stride,
                                                            uint8_t* __restrict__ tile_min,
                                                            uint8_t* __restrict__ tile_max,
                                                            NoAllocScratch* __restrict__ sc,
                                                            uint32_t* __restrict__ frame_out) {
    __shared__ uint32_t s_span[256];
    __shared__ uint32_t s_mean[64];
    __shared__ int s_lo, s_hi, s_last;
    __shared__ float s_wb[64], s_sb[64], s_tot[2];
    __shared__ float s_best_val[2];
    __shared__ int s_best_idx[2];

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

    const int y0 = ty * kTile;
    const int rows = min(kTile, H - y0);
    int lo = INT_MAX, hi = -1;
    for (int tx = tid; tx < tw; tx += blockDim.x) {
        const int x0 = tx * kTile;
        const int cols = min(kTile, W - x0);
        const uint8_t* p = gray + static_cast<int64_t>(y0) * stride + x0;
        uint32_t mn = 255u, mx = 0u, sum = 0u;
        for (int r = 0; r < rows; ++r) {
            for (int c = 0; c < cols; ++c) {
                const uint32_t v = p[r * stride + c];
                mn = min(mn, v);
                mx = max(mx, v);
                sum += v;
            }
        }
        const uint32_t count = static_cast<uint32_t>(rows * cols);
        const uint32_t mean = (sum + count / 2) / count;
        tile_min[ty * tw + tx] = static_cast<uint8_t>(mn);
        tile_max[ty * tw + tx] = static_cast<uint8_t>(mx);
        atomicAdd(&s_span[(mx - mn) & 0xffu], 1u);
        atomicAdd(&s_mean[mean >> 2], 1u);
        if (static_cast<int>(mx - mn) >= kMinTileContrast) {
            lo = min(lo, tx);
            hi = max(hi, tx);
        }
    }
    lo = __reduce_min_sync(kFull, lo);
    hi = __reduce_max_sync(kFull, hi);
    if ((tid & 31) == 0 && hi >= 0) {
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

    const int lane = tid & 31;
    if (tid < 32) {
        uint32_t v[8];
        uint32_t local = 0;
        for (int k = 0; k < 8; ++k) {
            v[k] = __ldcg(&sc->span_hist[lane * 8 + k]);
            local += v[k];
        }
        uint32_t incl = local;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t n = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += n;
        }
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        uint32_t span = 0;
        if (total > 0) {
            const uint32_t target = total / 4;
            uint32_t seen = incl - local;
            int hit = -1;
            for (int k = 0; k < 8; ++k) {
                seen += v[k];
                if (hit < 0 && seen > target) hit = lane * 8 + k;
            }
            const unsigned any = __ballot_sync(kFull, hit >= 0);
            span = static_cast<uint32_t>(__shfl_sync(kFull, hit, __ffs(any) - 1));
        }
        if (lane == 0) frame_out[0] = span;
    } else if (tid == 32) {
        float total = 0.0f, sum = 0.0f;
        for (int i = 0; i < 64; ++i) {
            const float m = static_cast<float>(__ldcg(&sc->mean_hist[i]));
            total += m;
            sum += static_cast<float>(i) * m;
            s_wb[i] = total;
            s_sb[i] = sum;
        }
        s_tot[0] = total;
        s_tot[1] = sum;
    }
    __syncthreads();
    if (tid < 64) {
        const float total = s_tot[0], sum = s_tot[1];
        const float wb = s_wb[tid];
        const float wa = total - wb;
        float between = -2.0f;
        if (total > 0.0f && wb > 0.0f && wa > 0.0f) {
            const float sb = s_sb[tid];
            const float mean_below = sb / wb;
            const float mean_above = (sum - sb) / wa;
            const float delta = mean_below - mean_above;
            between = wb * wa * delta * delta;
        }
        int idx = tid;
        for (int off = 16; off > 0; off >>= 1) {
            const float ov = __shfl_down_sync(kFull, between, off);
            const int oi = __shfl_down_sync(kFull, idx, off);
            if (ov > between || (ov == between && oi < idx)) {
                between = ov;
                idx = oi;
            }
        }
        if (lane == 0) {
            s_best_val[tid >> 5] = between;
            s_best_idx[tid >> 5] = idx;
        }
    }
    __syncthreads();
    if (tid == 0) {
        float best = s_best_val[0];
        int idx = s_best_idx[0];
        if (s_best_val[1] > best) {
            best = s_best_val[1];
            idx = s_best_idx[1];
        }
        frame_out[1] = static_cast<uint32_t>((best > -1.0f ? idx : 0) * 4 + 2);
        const uint32_t te = __ldcg(&sc->top_enc), be = __ldcg(&sc->bottom_enc);
        uint32_t roi = 0;
        if (be > 0) {
            const int top = th - static_cast<int>(te);
            const int bottom = static_cast<int>(be) - 1;
            roi = static_cast<uint32_t>(min(bottom + 1, th - 1) - max(top - 1, 0) + 1);
        }
        frame_out[2] = roi;
    }
}

// Device address of g_noalloc_scratch, looked up once per device.
constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
void* g_scratch_address[kMaxDevices] = {};

int32_t scratch_address(void** out) {
    int device = -1;
    cudaError_t st = cudaGetDevice(&device);
    if (st != cudaSuccess || device < 0 || device >= kMaxDevices) {
        set_last_error("bd_tile_stats_device_noalloc: no usable current CUDA device");
        return BD_ERROR_CUDA;
    }
    const std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[device]) {
        void* ptr = nullptr;
        st = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (st != cudaSuccess || !ptr) {
            cudaGetLastError();
            set_last_error("bd_tile_stats_device_noalloc: cudaGetSymbolAddress failed for the "
                           "scratch array");
            return BD_ERROR_CUDA;
        }
        g_scratch_address[device] = ptr;
    }
    *out = g_scratch_address[device];
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
    cudaError_t st = cudaMemsetAsync(scratch, 0, sizeof(NoAllocScratch), s);
    if (st == cudaSuccess) {
        const int tile_h = (height + kTile - 1) / kTile;
        k_tile_stats_noalloc<<<tile_h, 256, 0, s>>>(gray_device, width, height, stride,
                                                    tile_min_device, tile_max_device,
                                                    static_cast<NoAllocScratch*>(scratch),
                                                    frame_device);
        st = cudaGetLastError();
    }
    if (st != cudaSuccess) {
        cudaGetLastError();
        set_last_error(cudaGetErrorString(st));
        return BD_ERROR_CUDA;
    }
    return BD_OK;
}
