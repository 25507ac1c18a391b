// The whole pipeline of a batch as one persistent launch.
//
// Instead of one launch per stage (k_front.cu, k_quad.cu, k_finalize.cu),
// the CTAs of k_persistent pull work items from a queue in device memory,
// one (frame, stage, unit) at a time, and run the stage's device function on
// it (stage_front.cuh, stage_quad.cuh, stage_finalize.cuh):
//
//   STATS  unit = stats_rows tile rows   (the queue's first positions)
//   BIN    unit = band (8 pixel rows)
//   MERGE  unit = band
//   REGION unit = band
//   CAND   unit = band
//   FIT    unit = one big candidate (whole CTA), or a worker CTA whose warps
//          take (small candidate, family) pairs of the frame one at a time
//          from a per-frame counter until none is left
//   FINAL  unit = one family of the frame
//
// Per frame and stage a counter in FrameState counts finished units; the
// CTA that finishes a frame's last unit of a stage publishes that frame's
// units of the next stage.  So a frame's stages follow one another as soon
// as its own previous stage is done, while other frames are still in
// earlier stages, and no stage waits for a launch boundary.
//
// Waiting.  A CTA claims queue positions in order (one atomic counter) and
// waits until its position's item is published.  Items are published only
// by CTAs that are running an item, so a waiting CTA never waits for a CTA
// that has not started, and the launch needs no co-residency guarantee.
// Every wait is bounded (PersistParams::timeout_ns of %globaltimer): when it
// runs out the CTA records kQueueTimeout in the queue status and in every
// frame's result header, tells every CTA to leave, and returns.
//
// Memory ordering.  A CTA ends a unit with bar.sync, then one thread's
// __threadfence() and atomicAdd on the stage counter; the CTA that sees the
// last count fences again before it reads what the others wrote and before
// it publishes items.  A claiming thread fences after it sees its item and
// before bar.sync releases the CTA.  This file is compiled with
// -Xptxas -dlcm=cg, so plain loads of pipeline buffers are served by L2 and
// never by a stale L1 line; the frame itself is read through the read-only
// path (__ldg), which is safe because nothing writes it during the launch.

#include "stage_finalize.cuh"
#include "stage_front.cuh"
#include "stage_quad.cuh"

namespace bdgb {

namespace {

enum ItemKind : uint32_t {
    kStats = 1, kBin = 2, kMerge = 3, kRegion = 4, kCand = 5, kFitBig = 6, kFitSmall = 7, kFinal = 8
};

__host__ __device__ constexpr uint32_t encode_item(uint32_t kind, uint32_t frame, uint32_t index) {
    return (kind << 28) | (frame << 22) | index;
}

constexpr int kPersistThreads = 256;
constexpr int kSmallPerUnit = kPersistThreads / 32;  // (candidate, family) pairs per small-fit worker

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ uint32_t load_volatile(const uint32_t* p) {
    return *reinterpret_cast<const volatile uint32_t*>(p);
}

// Queue positions [0, seed): every frame's statistics units, in frame order.
__device__ __forceinline__ uint32_t seed_item(const BatchDesc* b, uint32_t pos) {
    int lo = 0, hi = b->frames - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b->stats_prefix[mid] <= static_cast<int>(pos)) lo = mid; else hi = mid - 1;
    }
    return encode_item(kStats, static_cast<uint32_t>(lo), pos - static_cast<uint32_t>(b->stats_prefix[lo]));
}

// Gives up the launch: the status says why, every frame's header carries it
// (FrameResultHeader::pad), and every CTA leaves at its next claim.
__device__ void abandon(const BatchDesc* b, WorkQueue* q, uint32_t why) {
    atomicOr(&q->status, why);
    for (int f = 0; f < b->frames; ++f) atomicOr(&b->f[f].result->pad, why);
    __threadfence();
    atomicExch(&q->finished, 1u);
}

// Thread 0: the next item (0: leave).  Bounded wait for an unpublished slot.
__device__ uint32_t claim(const BatchDesc* b, WorkQueue* q, uint32_t seed, uint64_t timeout_ns) {
    if (load_volatile(&q->finished)) return 0;
    const uint32_t pos = atomicAdd(&q->head, 1u);
    if (pos < seed) return seed_item(b, pos);
    const uint32_t slot = pos - seed;
    const uint64_t t0 = global_ns();
    for (unsigned backoff = 16;;) {
        if (slot < b->queue_capacity) {
            const uint32_t v = load_volatile(&q->items[slot]);
            if (v) {
                __threadfence();
                return v;
            }
        }
        if (load_volatile(&q->finished)) return 0;
        if (global_ns() - t0 > timeout_ns) {
            abandon(b, q, kQueueTimeout);
            return 0;
        }
        __nanosleep(backoff);
        backoff = min(backoff * 2, 256u);
    }
}

// Publishes `count` items (kind, frame, 0..count-1).  Called by the whole
// CTA after the unit's writes; `skip` (the stall test hook) withholds item 0.
__device__ void publish(const BatchDesc* b, WorkQueue* q, uint32_t kind, int fi, uint32_t count,
                        bool skip, uint32_t* s_base) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const uint32_t base = atomicAdd(&q->reserve, count);
        if (base + count > b->queue_capacity) {
            abandon(b, q, kQueueOverflow);
            *s_base = kNone;
        } else {
            *s_base = base;
        }
    }
    __syncthreads();
    const uint32_t base = *s_base;
    if (base == kNone) return;
    __threadfence();
    for (uint32_t i = threadIdx.x; i < count; i += blockDim.x) {
        if (skip && i == 0) continue;
        *reinterpret_cast<volatile uint32_t*>(&q->items[base + i]) =
            encode_item(kind, static_cast<uint32_t>(fi), i);
    }
}

// Counts a finished unit; true in the CTA that finished the last of `total`.
__device__ bool finish_unit(uint32_t* counter, uint32_t total, int* s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        *s_flag = atomicAdd(counter, 1u) == total - 1u;
    }
    __syncthreads();
    const bool last = *s_flag != 0;
    if (last) __threadfence();
    return last;
}

// Fit units of a frame after its candidates were placed: one per big
// candidate, one worker CTA per eight (small candidate, family) pairs, or
// straight to finalize when there is nothing to fit.
__device__ void publish_fit(const BatchDesc* b, WorkQueue* q, int fi, uint32_t n_big, uint32_t n_small,
                            uint32_t* s_base) {
    const FrameDesc& d = b->f[fi];
    const uint32_t pairs = n_small * static_cast<uint32_t>(__popc(d.families & 3u));
    const uint32_t small_units = (pairs + kSmallPerUnit - 1) / kSmallPerUnit;
    if (threadIdx.x == 0) d.state->fit_units = n_big + small_units;
    if (n_big + small_units == 0) {
        publish(b, q, kFinal, fi, 2, false, s_base);
        return;
    }
    if (n_big) publish(b, q, kFitBig, fi, n_big, false, s_base);
    if (small_units) publish(b, q, kFitSmall, fi, small_units, false, s_base);
}

// Shared memory: the stages' structs overlay one dynamic region.
struct PersistStatic {
    uint32_t item;
    uint32_t base;
    int flag;
    float uv[2][8];
};

__global__ void __launch_bounds__(kPersistThreads, 3)
k_persistent(const BatchDesc* __restrict__ b, const FrameIO* __restrict__ io, WorkQueue* q, int band_cap,
             int bits_words, int row_cap_max, int split_px, uint32_t seed, PersistParams pp) {
    extern __shared__ __align__(16) uint32_t s_dyn[];
    __shared__ PersistStatic ps;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    if (tid < 16) {
        const int fam = tid >> 3, c = tid & 7;
        ps.uv[fam][c] = (c + 0.5f) / static_cast<float>(family_dim(fam));
    }
    // Probe direction of this lane (reference :1134-1170).
    float ux, uy;
    {
        const float angle = 6.28318530718f * static_cast<float>(lane) / static_cast<float>(kFitDirections);
        bdmath::sincos(angle, &uy, &ux);
    }
    // Regions of the overlay that follow a stage's struct.
    constexpr size_t kBinDyn = (sizeof(BinSmem) + 15) / 16 * 16;
    constexpr size_t kCandDyn = (sizeof(CandSmem) + 15) / 16 * 16;
    unsigned char* dyn = reinterpret_cast<unsigned char*>(s_dyn);

    for (;;) {
        if (tid == 0) ps.item = claim(b, q, seed, pp.timeout_ns);
        __syncthreads();
        const uint32_t item = ps.item;
        if (item == 0) break;
        const uint32_t kind = item >> 28;
        const int fi = static_cast<int>((item >> 22) & 63u);
        const uint32_t idx = item & 0x3fffffu;
        const FrameDesc& d = b->f[fi];
        FrameState* st = d.state;
        const uint32_t th = static_cast<uint32_t>(d.tile_h);
        switch (kind) {
            case kStats: {
                const uint32_t units = static_cast<uint32_t>(b->stats_prefix[fi + 1] - b->stats_prefix[fi]);
                const bool used = io[fi].gray != nullptr;
                if (used) stage_stats(b, io, fi, static_cast<int>(idx), *reinterpret_cast<StatsSmem*>(dyn));
                if (finish_unit(&st->done_stats, units, &ps.flag)) {
                    if (used) {
                        publish(b, q, kBin, fi, th, pp.stall_frame == fi, &ps.base);
                    } else {
                        publish(b, q, kFinal, fi, 2, false, &ps.base);  // unused slot: empty results
                    }
                }
                break;
            }
            case kBin:
                stage_binarize(b, io, fi, static_cast<int>(idx), band_cap, bits_words,
                               *reinterpret_cast<BinSmem*>(dyn), reinterpret_cast<uint32_t*>(dyn + kBinDyn));
                if (finish_unit(&st->done_bin, th, &ps.flag)) publish(b, q, kMerge, fi, th, false, &ps.base);
                break;
            case kMerge:
                stage_merge(b, fi, static_cast<int>(idx), row_cap_max, s_dyn);
                if (finish_unit(&st->done_merge, th, &ps.flag)) publish(b, q, kRegion, fi, th, false, &ps.base);
                break;
            case kRegion:
                stage_region(b, fi, static_cast<int>(idx));
                if (finish_unit(&st->done_region, th, &ps.flag)) publish(b, q, kCand, fi, th, false, &ps.base);
                break;
            case kCand: {
                CandSmem& cs = *reinterpret_cast<CandSmem*>(dyn);
                if (stage_cand(b, fi, static_cast<int>(idx), split_px, cs,
                               reinterpret_cast<uint32_t*>(dyn + kCandDyn))) {
                    __syncthreads();
                    publish_fit(b, q, fi, cs.nbig, cs.nsmall, &ps.base);
                }
                break;
            }
            case kFitBig:
                fit_big_item(b, io, fi, static_cast<int>(idx), ux, uy, ps.uv, *reinterpret_cast<BigSmem*>(dyn));
                if (finish_unit(&st->done_fit, __ldcg(&st->fit_units), &ps.flag)) {
                    publish(b, q, kFinal, fi, 2, false, &ps.base);
                }
                break;
            case kFitSmall: {
                // Every warp takes the frame's next pair until none is left,
                // so a worker ends within one pair of the others.
                const int nfam = __popc(d.families & 3u);
                const uint32_t pairs = __ldcg(&st->n_small) * static_cast<uint32_t>(nfam);
                for (;;) {
                    uint32_t pair = 0;
                    if (lane == 0) pair = atomicAdd(&st->small_next, 1u);
                    pair = __shfl_sync(kFull, pair, 0);
                    if (pair >= pairs) break;
                    const int k = static_cast<int>(pair) / nfam;
                    fit_small_item(b, io, fi, k, static_cast<int>(pair) - k * nfam, ux, uy, ps.uv,
                                   reinterpret_cast<QuadSmem*>(dyn)[warp], lane);
                }
                if (finish_unit(&st->done_fit, __ldcg(&st->fit_units), &ps.flag)) {
                    publish(b, q, kFinal, fi, 2, false, &ps.base);
                }
                break;
            }
            case kFinal:
                stage_finalize(b, fi, static_cast<int>(idx), *reinterpret_cast<FinalSmem*>(dyn));
                if (finish_unit(&st->done_final, 2u, &ps.flag) && tid == 0) {
                    if (atomicAdd(&q->frames_done, 1u) == static_cast<uint32_t>(b->frames) - 1u) {
                        atomicExch(&q->finished, 1u);
                    }
                }
                break;
            default:
                if (tid == 0) abandon(b, q, kQueueOverflow);
                break;
        }
        __syncthreads();  // the overlay is reused by the next item
    }
}

size_t persistent_smem_bytes(int band_cap, int bits_words, int row_cap_max, int tile_h_max) {
    constexpr size_t kBinDyn = (sizeof(BinSmem) + 15) / 16 * 16;
    constexpr size_t kCandDyn = (sizeof(CandSmem) + 15) / 16 * 16;
    size_t bytes = sizeof(StatsSmem);
    bytes = std::max(bytes, kBinDyn + band_smem_bytes(band_cap, bits_words));
    bytes = std::max(bytes, 2 * static_cast<size_t>(row_cap_max) * sizeof(uint32_t));
    bytes = std::max(bytes, kCandDyn + (static_cast<size_t>(tile_h_max) + 1) * sizeof(uint32_t));
    bytes = std::max(bytes, kSmallPerUnit * sizeof(QuadSmem));
    bytes = std::max(bytes, sizeof(BigSmem));
    bytes = std::max(bytes, sizeof(FinalSmem));
    return (bytes + 15) / 16 * 16;
}

}  // namespace

int prepare_persistent() {
    // The largest overlay: band cap 2048 on the widest frame, tallest frame.
    const size_t most = persistent_smem_bytes(kMaxBandCap, BD_MAX_WIDTH / 32, BD_MAX_WIDTH / 2 + 2,
                                              BD_MAX_HEIGHT / kTile);
    return cudaFuncSetAttribute(k_persistent, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                static_cast<int>(most)) == cudaSuccess
               ? 0
               : -1;
}

void enqueue_persistent(const BatchDesc* dd, const BatchDesc& hd, const FrameIO* io, WorkQueue* queue,
                        void* stream_ptr, const LaunchConfig& lc, int sm_count, const PersistParams& pp) {
    cudaStream_t s = static_cast<cudaStream_t>(stream_ptr);
    int words_max = 1, row_cap_max = 1, th_max = 1;
    for (int f = 0; f < hd.frames; ++f) {
        words_max = std::max(words_max, hd.f[f].words);
        row_cap_max = std::max(row_cap_max, hd.f[f].row_cap);
        th_max = std::max(th_max, hd.f[f].tile_h);
    }
    const size_t smem = persistent_smem_bytes(lc.band_cap, words_max, row_cap_max, th_max);
    int grid = lc.persist_ctas;
    if (grid <= 0) {
        int per_sm = 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_persistent, kPersistThreads, smem);
        grid = std::max(1, per_sm) * sm_count;
    }
    k_persistent<<<grid, kPersistThreads, smem, s>>>(dd, io, queue, lc.band_cap, words_max, row_cap_max,
                                                     lc.quad_split,
                                                     static_cast<uint32_t>(hd.stats_ctas), pp);
}

}  // namespace bdgb
