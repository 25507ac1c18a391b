// Stage 7 as a device function of one CTA: de-duplication, sort by id and
// the result records of one (frame, family).  k_finalize (k_finalize.cu)
// and the persistent kernel (k_persistent.cu) both call it.
#pragma once

#include "kernels_common.cuh"
#include "kernels.cuh"

namespace bdgb {
namespace {

struct FinalSmem {
    DecodeOut in[kMaxDetectionsCap];
    DecodeOut out[kMaxDetectionsCap];
    float cx[kMaxDetectionsCap], cy[kMaxDetectionsCap];
    float h[kMaxDetectionsCap][9];     // homography of each compacted detection
    int out_in[kMaxDetectionsCap];     // compacted index of each kept detection
    uint32_t warp[kFinalThreads / 32];
    int count, kept;
};

// Image homography of a detection's corners (reference host
// fill_homography :1739-1774, FP64 as there), one detection per thread of
// the finalizing CTA.
__device__ void fill_homography(const float corners[8], float H[9]) {
    const double x0 = corners[0], y0 = corners[1];
    const double x1 = corners[2], y1 = corners[3];
    const double x2 = corners[4], y2 = corners[5];
    const double x3 = corners[6], y3 = corners[7];
    const double dx1 = x1 - x2, dx2 = x3 - x2;
    const double dx3 = x0 - x1 + x2 - x3;
    const double dy1 = y1 - y2, dy2 = y3 - y2;
    const double dy3 = y0 - y1 + y2 - y3;
    double g = 0.0, h = 0.0;
    const double det = dx1 * dy2 - dx2 * dy1;
    if (fabs(det) > 1e-12) {
        g = (dx3 * dy2 - dx2 * dy3) / det;
        h = (dx1 * dy3 - dx3 * dy1) / det;
    }
    const double a = x1 - x0 + g * x1;
    const double bb = x3 - x0 + h * x3;
    const double dd = y1 - y0 + g * y1;
    const double e = y3 - y0 + h * y3;
    const double w = g + h + 2.0;
    const double inv = (fabs(w) > 1e-12) ? 1.0 / w : 0.0;
    H[0] = static_cast<float>(a * inv);
    H[1] = static_cast<float>(bb * inv);
    H[2] = static_cast<float>((a + bb + 2.0 * x0) * inv);
    H[3] = static_cast<float>(dd * inv);
    H[4] = static_cast<float>(e * inv);
    H[5] = static_cast<float>((dd + e + 2.0 * y0) * inv);
    H[6] = static_cast<float>(g * inv);
    H[7] = static_cast<float>(h * inv);
    H[8] = static_cast<float>(w * inv);
}

// ===========================================================================
// 9. Finalize one (frame, family): detections in candidate order (first
//    max_detections), de-duplication, stable sort by id, homography
//    (reference k_finalize :1542-1601, host fill_homography :1739-1774 --
//    FP64 here as there).  Expects blockDim.x == kFinalThreads.
// ===========================================================================
__device__ __forceinline__ void stage_finalize(const BatchDesc* __restrict__ b, int fi, int fam,
                                               FinalSmem& sm) {
    DecodeOut* s_in = sm.in;
    DecodeOut* s_out = sm.out;
    float* s_cx = sm.cx;
    float* s_cy = sm.cy;
    uint32_t* s_warp = sm.warp;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
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
    if (tid == 0) sm.count = 0;
    __syncthreads();
    // Ordered compaction of the decoded candidates.
    for (int c = 0; c < n; c += kFinalThreads) {
        const int i = c + tid;
        const bool ok = i < n && dec[i].id >= 0;
        const unsigned bal = __ballot_sync(kFull, ok);
        if (lane == 0) s_warp[warp] = __popc(bal);
        __syncthreads();
        int before = sm.count;
        for (int w2 = 0; w2 < warp; ++w2) before += static_cast<int>(s_warp[w2]);
        const int pos = before + __popc(bal & lanemask_lt());
        if (ok && pos < maxd) {
            s_in[pos] = dec[i];
        }
        __syncthreads();
        if (tid == 0) {
            int add = 0;
            for (int w2 = 0; w2 < kFinalThreads / 32; ++w2) add += static_cast<int>(s_warp[w2]);
            sm.count = sm.count + add;
        }
        __syncthreads();
        if (sm.count >= maxd) break;
    }
    const int m = min(sm.count, maxd);
    // De-duplication in arrival order, one warp; the other warps meanwhile
    // form the homography of every compacted detection (FP64 is slow, and
    // the kept ones are among them).
    if (warp > 0) {
        for (int i = tid - 32; i < m; i += kFinalThreads - 32) fill_homography(s_in[i].corners, sm.h[i]);
    } else {
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
                        sm.out_in[duplicate] = i;
                        s_cx[duplicate] = cx;
                        s_cy[duplicate] = cy;
                    }
                } else if (kept < maxd) {
                    s_out[kept] = dd;
                    sm.out_in[kept] = i;
                    s_cx[kept] = cx;
                    s_cy[kept] = cy;
                }
            }
            if (duplicate < 0 && kept < maxd) ++kept;
            __syncwarp();
        }
        if (lane == 0) sm.kept = kept;
    }
    __syncthreads();
    const int kept = sm.kept;
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
        for (int k = 0; k < 9; ++k) r.homography[k] = sm.h[sm.out_in[i]][k];
        dets[rank] = r;
    }
    if (tid == 0) hdr->found[fam] = static_cast<uint32_t>(kept);
}

}  // namespace
}  // namespace bdgb
