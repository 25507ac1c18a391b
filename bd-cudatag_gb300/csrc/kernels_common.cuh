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

__device__ __forceinline__ uint32_t uf_root_readonly(const uint32_t* parent, uint32_t x) {
    for (;;) {
        const uint32_t p = __ldcg(parent + x);
        if (p == x) return x;
        x = p;
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
