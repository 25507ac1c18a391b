// Device helpers shared by the kernel translation units of the batched
// pipeline (k_front.cu, k_quad.cu, k_finalize.cu): warp masks, the band
// lookup and the union-find with the reference's smallest-slot invariant.
#pragma once

#include <cuda_runtime.h>

#include <cfloat>
#include <climits>
#include <algorithm>
#include <cstdint>

#include "detmath.h"
#include "pipeline.cuh"

namespace bdgb {
namespace {


constexpr unsigned kFull = 0xffffffffu;

__device__ __forceinline__ int family_dim(int fam) { return fam == 0 ? 8 : 6; }

__device__ __forceinline__ int frame_of_band(const BatchDesc* __restrict__ b, int band) {
    int lo = 0, hi = b->frames - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (b->band_prefix[mid] <= band) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// A candidate whose bounding box has a side above `split_px` pixels is fitted
// and decoded by a whole CTA (k_fit_decode_big); 0 turns the split off.
__device__ __forceinline__ bool big_candidate(uint4 bb, int split_px) {
    return split_px > 0 && max(bb.z - bb.x, bb.w - bb.y) + 1 > static_cast<uint32_t>(split_px);
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    return (1u << (threadIdx.x & 31)) - 1u;
}

// 4 bits, bit k = (byte k of `pixels` > t).
__device__ __forceinline__ uint32_t white_bits4(uint32_t pixels, uint32_t t4) {
    const uint32_t gt = __vcmpgtu4(pixels, t4);  // 0xff per byte where pixel > t
    return (((gt >> 7) & 0x01010101u) * 0x10204080u) >> 28;
}

// ---------------------------------------------------------------------------
// Tile statistics (reference k_tile_stats :104-135): min, max and rounded
// mean of the 8x8 tiles of a frame.  One thread takes a pair of horizontally
// adjacent tiles, 16 pixels wide: with a 16-byte aligned frame and stride,
// full pairs are eight 128-bit loads issued together.
// ---------------------------------------------------------------------------
struct TileStat {
    uint32_t mn, mx, mean;
};

__device__ __forceinline__ uint32_t min_byte4(uint32_t v) {
    return min(min(v & 0xffu, (v >> 8) & 0xffu), min((v >> 16) & 0xffu, v >> 24));
}
__device__ __forceinline__ uint32_t max_byte4(uint32_t v) {
    return max(max(v & 0xffu, (v >> 8) & 0xffu), max((v >> 16) & 0xffu, v >> 24));
}

// Any tile: `rows` x `cols` pixels at p (rows, cols in 1..8).
__device__ __forceinline__ TileStat tile_stat_scalar(const uint8_t* __restrict__ p, int64_t stride,
                                                     int rows, int cols) {
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
    return {mn, mx, (sum + count / 2) / count};
}

// Tiles 2 * pair and 2 * pair + 1 of tile row ty; b.mn = 256 when the pair
// has one tile only (odd tile count).  vec16: gray and stride are multiples
// of 16 bytes.
__device__ __forceinline__ void tile_pair_stats(const uint8_t* __restrict__ gray, int64_t stride,
                                                int W, int H, int ty, int pair, bool vec16,
                                                TileStat* a, TileStat* b) {
    const int y0 = ty * kTile;
    const int x0 = pair * 2 * kTile;
    const int rows = min(kTile, H - y0);
    const uint8_t* p = gray + static_cast<int64_t>(y0) * stride + x0;
    if (vec16 && rows == kTile && x0 + 2 * kTile <= W) {
        uint4 v[kTile];
#pragma unroll
        for (int r = 0; r < kTile; ++r) v[r] = __ldg(reinterpret_cast<const uint4*>(p + r * stride));
        uint32_t amin = 0xffffffffu, amax = 0u, bmin = 0xffffffffu, bmax = 0u, asum = 0u, bsum = 0u;
#pragma unroll
        for (int r = 0; r < kTile; ++r) {
            amin = __vminu4(amin, __vminu4(v[r].x, v[r].y));
            amax = __vmaxu4(amax, __vmaxu4(v[r].x, v[r].y));
            bmin = __vminu4(bmin, __vminu4(v[r].z, v[r].w));
            bmax = __vmaxu4(bmax, __vmaxu4(v[r].z, v[r].w));
            asum = __dp4a(v[r].x, 0x01010101u, asum);
            asum = __dp4a(v[r].y, 0x01010101u, asum);
            bsum = __dp4a(v[r].z, 0x01010101u, bsum);
            bsum = __dp4a(v[r].w, 0x01010101u, bsum);
        }
        *a = {min_byte4(amin), max_byte4(amax), (asum + 32u) >> 6};
        *b = {min_byte4(bmin), max_byte4(bmax), (bsum + 32u) >> 6};
        return;
    }
    *a = tile_stat_scalar(p, stride, rows, min(kTile, W - x0));
    if (x0 + kTile < W) {
        *b = tile_stat_scalar(p + kTile, stride, rows, min(kTile, W - x0 - kTile));
    } else {
        *b = {256u, 0u, 0u};
    }
}

// Frame references from the span and mean histograms (reference
// k_tile_reference :174-230): [0] the lower quartile of the tile spans, [1]
// the Otsu level of the tile means.  Called by every thread of a CTA of at
// least 64 threads.
//
// The reference sums the Otsu prefixes sequentially in FP32.  Every partial
// sum is an integer no larger than sum = sum_i i * hist[i]; while that is
// below 2^24 every one is exact in FP32, so an integer scan converted to
// float gives the same bits in any order.  That holds for every frame of up
// to 266,305 tiles (63 * tiles < 2^24: 4096 x 4096 and below); larger frames
// take the sequential loop.
struct RefSmem {
    uint32_t mh[64];
    float wb[64], sb[64];
    float tot[2];
    float best_val[2];
    int best_idx[2];
};

__device__ __forceinline__ void frame_references(const uint32_t* span_hist, const uint32_t* mean_hist,
                                                 RefSmem& sm, uint32_t* span_out, uint32_t* otsu_out) {
    const int tid = threadIdx.x, lane = tid & 31;
    if (tid < 32) {
        // Lower quartile: first bin whose cumulative count exceeds total / 4.
        uint32_t v[8];
        uint32_t local = 0;
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            v[k] = __ldcg(&span_hist[lane * 8 + k]);
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
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                seen += v[k];
                if (hit < 0 && seen > target) hit = lane * 8 + k;
            }
            const unsigned any = __ballot_sync(kFull, hit >= 0);
            span = static_cast<uint32_t>(__shfl_sync(kFull, hit, __ffs(any) - 1));
        }
        if (lane == 0) *span_out = span;
    } else if (tid < 64) {
        // Otsu prefixes: lane l holds bins 2l and 2l + 1.
        const uint32_t m0 = __ldcg(&mean_hist[2 * lane]), m1 = __ldcg(&mean_hist[2 * lane + 1]);
        const uint32_t cnt = m0 + m1;
        const uint32_t wsum = static_cast<uint32_t>(2 * lane) * m0 + static_cast<uint32_t>(2 * lane + 1) * m1;
        uint32_t ic = cnt, is = wsum;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t nc = __shfl_up_sync(kFull, ic, off);
            const uint32_t ns = __shfl_up_sync(kFull, is, off);
            if (lane >= off) {
                ic += nc;
                is += ns;
            }
        }
        const uint32_t S = __shfl_sync(kFull, is, 31);
        if (S < (1u << 24)) {
            const uint32_t c0 = ic - cnt + m0, s0 = is - wsum + static_cast<uint32_t>(2 * lane) * m0;
            sm.wb[2 * lane] = static_cast<float>(c0);
            sm.sb[2 * lane] = static_cast<float>(s0);
            sm.wb[2 * lane + 1] = static_cast<float>(ic);
            sm.sb[2 * lane + 1] = static_cast<float>(is);
            if (lane == 31) {
                sm.tot[0] = static_cast<float>(ic);
                sm.tot[1] = static_cast<float>(is);
            }
        } else {
            sm.mh[2 * lane] = m0;
            sm.mh[2 * lane + 1] = m1;
            __syncwarp();
            if (lane == 0) {
                float total = 0.0f, sum = 0.0f;
                for (int i = 0; i < 64; ++i) {
                    const float m = static_cast<float>(sm.mh[i]);
                    total += m;
                    sum += static_cast<float>(i) * m;
                    sm.wb[i] = total;
                    sm.sb[i] = sum;
                }
                sm.tot[0] = total;
                sm.tot[1] = sum;
            }
        }
    }
    __syncthreads();
    if (tid < 64) {
        // Between-class variance of every split; the first maximum wins.
        const float total = sm.tot[0], sum = sm.tot[1];
        const float wb = sm.wb[tid];
        const float wa = total - wb;
        float between = -2.0f;
        if (total > 0.0f && wb > 0.0f && wa > 0.0f) {
            const float sb = sm.sb[tid];
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
            sm.best_val[tid >> 5] = between;
            sm.best_idx[tid >> 5] = idx;
        }
    }
    __syncthreads();
    if (tid == 0) {
        float best = sm.best_val[0];
        int idx = sm.best_idx[0];
        if (sm.best_val[1] > best) {
            best = sm.best_val[1];
            idx = sm.best_idx[1];
        }
        *otsu_out = static_cast<uint32_t>((best > -1.0f ? idx : 0) * 4 + 2);
    }
}

// ROI tile rows of a frame from its first / last contrasting tile row (the
// encoded maxima): every row between them, one row of halo each side
// (reference :314-330, :2117).
__device__ __forceinline__ uint32_t roi_tile_rows(uint32_t top_enc, uint32_t bottom_enc, int tile_h) {
    if (bottom_enc == 0) return 0;
    const int top = tile_h - static_cast<int>(top_enc);
    const int bottom = static_cast<int>(bottom_enc) - 1;
    return static_cast<uint32_t>(min(bottom + 1, tile_h - 1) - max(top - 1, 0) + 1);
}

// ---------------------------------------------------------------------------
// Union-find with the reference's invariant: a label only ever moves to a
// smaller slot id, so the root of a component is its smallest run slot
// (gpu_detector.cu:398-421).
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t uf_find(uint32_t* parent, uint32_t x) {
    for (;;) {
        const uint32_t p = parent[x];
        if (p == x) return x;
        const uint32_t gp = parent[p];
        parent[x] = gp;
        x = gp;
    }
}

// Root of x once every union is done, halving the path as it walks: each
// node passed is pointed at its grandparent, so walks of the same chain that
// start later (from other bands) take fewer steps.  The halving link is an
// atomicMin, so it never raises a link that another walker has already set
// to the component's root (the smallest slot of the component).
__device__ __forceinline__ uint32_t uf_root_halving(uint32_t* parent, uint32_t x) {
    for (;;) {
        const uint32_t p = __ldcg(parent + x);
        if (p == x) return x;
        const uint32_t gp = __ldcg(parent + p);
        if (gp == p) return p;
        atomicMin(parent + x, gp);
        x = gp;
    }
}

// Roots of *a and *b, the two chains walked in lockstep (path halving on
// both, as uf_find) so that their loads are in flight together.
__device__ __forceinline__ void uf_find2(uint32_t* parent, uint32_t* a, uint32_t* b) {
    uint32_t x = *a, y = *b;
    for (;;) {
        const uint32_t px = parent[x], py = parent[y];
        const bool rx = px == x, ry = py == y;
        if (rx && ry) break;
        const uint32_t gx = rx ? px : parent[px];
        const uint32_t gy = ry ? py : parent[py];
        if (!rx) {
            parent[x] = gx;
            x = gx;
        }
        if (!ry) {
            parent[y] = gy;
            y = gy;
        }
    }
    *a = x;
    *b = y;
}

__device__ __forceinline__ void uf_union(uint32_t* parent, uint32_t a, uint32_t b) {
    uf_find2(parent, &a, &b);
    while (a != b) {
        if (a > b) {
            const uint32_t t = a;
            a = b;
            b = t;
        }
        const uint32_t old = atomicMin(&parent[b], a);
        // b was still a root (now under a), or already under a: joined.
        if (old == b || old == a) break;
        b = uf_find(parent, old);
    }
}

}  // namespace
}  // namespace bdgb
