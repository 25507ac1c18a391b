// Quad fit and decode of the candidates as device functions: hull, four
// corners, edge refinement, the four rotations of each quad; one (small
// candidate, family) item per warp (fit_small_item)
// or one big candidate per CTA (fit_big_item).  The per-stage kernels
// (k_quad.cu) and the persistent kernel (k_persistent.cu) both call them.  All FP32
// arithmetic follows the reference expressions term by term and is compiled
// with -fmad=false; transcendentals come from detmath.h.  With the oracle
// built the same way, corners and margins match it bit for bit.

#pragma once

#include "kernels_common.cuh"
#include "kernels.cuh"
#include "families_data.inc"

namespace bdgb {
namespace {

__device__ const uint64_t d_codes36h11[BD_CODEWORDS_36H11_COUNT] = {BD_CODEWORDS_36H11};
__device__ const uint64_t d_codes16h5[BD_CODEWORDS_16H5_COUNT] = {BD_CODEWORDS_16H5};

// ===========================================================================
// 7. Quad fit (reference k_fit_quads :1081-1241 and helpers :659-1076).
// ===========================================================================
__device__ __forceinline__ uint32_t pack_point(int x, int y) {
    return (static_cast<uint32_t>(x) & 0xffffu) | (static_cast<uint32_t>(y) << 16);
}

// hull_to_quad (reference :736-831) run by one warp: lane i holds hull
// vertex i; each round drops the vertex whose triangle with its neighbours
// has the smallest area (first index on ties, as the reference's strict <),
// found with a warp arg-min instead of a serial scan.  The remaining checks
// run on lane 0 with the reference's expressions.  Returns the result in all
// lanes.
__device__ bool hull_to_quad_warp(const uint32_t* hull, int count, float quad[4][2], int lane) {
    if (count < 4 || count > kMaxHullVertices || count > 32) return false;
    float vx = lane < count ? static_cast<float>(hull[lane] & 0xffffu) : 0.0f;
    float vy = lane < count ? static_cast<float>(hull[lane] >> 16) : 0.0f;
    while (count > 4) {
        // Cyclic neighbours (lanes >= count compute garbage that is unused).
        const int prev = lane == 0 ? count - 1 : lane - 1;
        const int next = lane + 1 >= count ? 0 : lane + 1;
        const float pvx = __shfl_sync(kFull, vx, prev), pvy = __shfl_sync(kFull, vy, prev);
        const float nvx = __shfl_sync(kFull, vx, next), nvy = __shfl_sync(kFull, vy, next);
        float area = FLT_MAX;
        if (lane < count) {
            const float ax = vx - pvx;
            const float ay = vy - pvy;
            const float bx = nvx - vx;
            const float by = nvy - vy;
            area = fabsf(ax * by - ay * bx) * 0.5f;
            if (!(area < FLT_MAX)) area = FLT_MAX;
        }
        // Areas are >= 0, so their bit patterns order like the values.
        const uint32_t key = __float_as_uint(area);
        const uint32_t best_key = __reduce_min_sync(kFull, key);
        if (best_key == __float_as_uint(FLT_MAX)) return false;
        const int idx = __ffs(__ballot_sync(kFull, lane < count && key == best_key)) - 1;
        const float sx = __shfl_down_sync(kFull, vx, 1), sy = __shfl_down_sync(kFull, vy, 1);
        if (lane >= idx) {
            vx = sx;
            vy = sy;
        }
        --count;
    }
    float qx[4], qy[4];
    for (int i = 0; i < 4; ++i) {
        qx[i] = __shfl_sync(kFull, vx, i);
        qy[i] = __shfl_sync(kFull, vy, i);
    }
    int ok = 0;
    if (lane == 0) {
        float* x = qx;
        float* y = qy;
        ok = 1;
        float area2 = 0.0f;
        for (int i = 0; i < 4; ++i) {
            const int j = (i + 1) & 3;
            area2 += x[i] * y[j] - x[j] * y[i];
        }
        if (fabsf(area2) < 24.0f) ok = 0;
        if (ok && area2 < 0.0f) {
            for (int i = 0; i < 2; ++i) {
                const float tx = x[i + 1], tyy = y[i + 1];
                x[i + 1] = x[3 - i];
                y[i + 1] = y[3 - i];
                x[3 - i] = tx;
                y[3 - i] = tyy;
            }
        }
        float min_side = FLT_MAX, max_side = 0.0f;
        for (int i = 0; ok && i < 4; ++i) {
            const int j = (i + 1) & 3;
            const float ex = x[j] - x[i];
            const float ey = y[j] - y[i];
            const float len = sqrtf(ex * ex + ey * ey);
            if (len < 4.0f) {
                ok = 0;
                break;
            }
            min_side = fminf(min_side, len);
            max_side = fmaxf(max_side, len);
            const int p = (i + 3) & 3;
            const float ax = x[i] - x[p];
            const float ay = y[i] - y[p];
            const float bx = x[j] - x[i];
            const float by = y[j] - y[i];
            if (ax * by - ay * bx <= 0.0f) {
                ok = 0;
                break;
            }
            const float dot = ax * bx + ay * by;
            const float n1 = sqrtf(ax * ax + ay * ay);
            const float n2 = sqrtf(bx * bx + by * by);
            if (n1 < 1e-3f || n2 < 1e-3f || fabsf(dot / (n1 * n2)) > 0.97f) {
                ok = 0;
                break;
            }
        }
        if (ok && max_side > 12.0f * min_side) ok = 0;
        if (ok) {
            const float cx = 0.25f * (x[0] + x[1] + x[2] + x[3]);
            const float cy = 0.25f * (y[0] + y[1] + y[2] + y[3]);
            for (int i = 0; i < 4; ++i) {
                const float dx = x[i] - cx;
                const float dy = y[i] - cy;
                const float len = sqrtf(dx * dx + dy * dy);
                if (len > 1e-3f) {
                    x[i] += dx / len * 0.65f;
                    y[i] += dy / len * 0.65f;
                }
            }
        }
    }
    ok = __shfl_sync(kFull, ok, 0);
    for (int i = 0; i < 4; ++i) {
        quad[i][0] = __shfl_sync(kFull, qx[i], 0);
        quad[i][1] = __shfl_sync(kFull, qy[i], 0);
    }
    return ok != 0;
}

__device__ __forceinline__ bool intersect_lines(const float li[4], const float lj[4], float* x,
                                                float* y) {
    const float det = li[2] * lj[3] - li[3] * lj[2];
    if (fabsf(det) < 0.2f) return false;
    const float di = li[2] * li[0] + li[3] * li[1];
    const float dj = lj[2] * lj[0] + lj[3] * lj[1];
    *x = (di * lj[3] - li[3] * dj) / det;
    *y = (li[2] * dj - di * lj[2]) / det;
    return true;
}

// Bilinear sample with the reference's bounds rule (sample_bilinear
// :833-849): -1 outside [0, width-1) x [0, height-1).  The address is
// clamped and the result selected instead of branching, which lets the loads
// of successive samples overlap (an early return here made the fit kernels
// about 8% slower); in-range values are computed with the reference's
// expression.  Used for the edge probes and the decode cells.
__device__ __forceinline__ float sample_ro(const uint8_t* __restrict__ image, int width, int height,
                                           int64_t stride, float x, float y) {
    const bool in = x >= 0.0f && y >= 0.0f && x < static_cast<float>(width - 1) &&
                    y < static_cast<float>(height - 1);
    const float xc = in ? x : 0.0f;
    const float yc = in ? y : 0.0f;
    const int ix = static_cast<int>(xc);
    const int iy = static_cast<int>(yc);
    const float fx = xc - static_cast<float>(ix);
    const float fy = yc - static_cast<float>(iy);
    const uint8_t* p = image + static_cast<int64_t>(iy) * stride + ix;
    const float a = __ldg(p);
    const float bb = __ldg(p + 1);
    const float c = __ldg(p + stride);
    const float dd = __ldg(p + stride + 1);
    const float v = (a * (1.0f - fx) + bb * fx) * (1.0f - fy) + (c * (1.0f - fx) + dd * fx) * fy;
    return in ? v : -1.0f;
}

__device__ __forceinline__ float rise_ro(const uint8_t* __restrict__ image, int width, int height,
                                         int64_t stride, float x, float y, float dx, float dy) {
    const float ahead = sample_ro(image, width, height, stride, x + dx * 0.7f, y + dy * 0.7f);
    const float behind = sample_ro(image, width, height, stride, x - dx * 0.7f, y - dy * 0.7f);
    if (ahead < 0.0f || behind < 0.0f) return 0.0f;
    return ahead - behind;
}

constexpr int kMaxProbes = kFitProbeHalf * 2 + 1;

// The four edge lines of one quad, fitted by one warp (reference
// fit_edge_line_warp :881-1016, which spends a warp per edge).  Lane l takes
// sample l % seg of edge base + l / seg, with seg = 8 when no edge has more
// than 8 samples (all four edges in one round) and 16 otherwise (two rounds
// of two edges).  A lane probes its whole profile into its own shared-memory
// row (kMaxProbes floats; the row stride is odd, so rows fall in different
// banks) and picks the peak exactly as the reference lane does.  An edge's
// moments are summed by a seg-lane shuffle tree: the reference sums them
// with a 32-lane tree over samples 0..15 and zeros above, whose first one
// (seg 16) or two (seg 8) levels only add +0.0, so adding +0.0 that many
// times and finishing within the segment gives the same bits.  Segment
// leaders fit the lines into lines[edge] / have[edge].
__device__ void fit_edges_warp(const float (*q)[2], const uint8_t* __restrict__ image, int width,
                               int height, int64_t stride, int dim, bool first_pass, int lane,
                               float* s_mags, float (*lines)[4], int* have) {
    int my_samples = 0;
    if (lane < 4) {
        const int bi = (lane + 1) & 3;
        const float ex = q[bi][0] - q[lane][0];
        const float ey = q[bi][1] - q[lane][1];
        const float len = sqrtf(ex * ex + ey * ey);
        if (len >= 8.0f) my_samples = min(max(static_cast<int>(len / 6.0f), 8), 16);
    }
    const int seg = __reduce_max_sync(kFull, static_cast<unsigned>(my_samples)) <= 8 ? 8 : 16;
    float* mags = s_mags + lane * kMaxProbes;
    const int seg_shift = seg == 8 ? 3 : 4;
    for (int base = 0; base < 4; base += 32 >> seg_shift) {
        const int edge = base + (lane >> seg_shift);
        const int sample = lane & (seg - 1);
        const int bi = (edge + 1) & 3;
        const float ax = q[edge][0], ay = q[edge][1];
        const float ex = q[bi][0] - ax;
        const float ey = q[bi][1] - ay;
        const float len = sqrtf(ex * ex + ey * ey);
        const bool edge_ok = len >= 8.0f;
        float mx = 0.0f, my = 0.0f, mxx = 0.0f, mxy = 0.0f, myy = 0.0f;
        int used = 0;
        if (edge_ok) {
            const float nx = ey / len;
            const float ny = -ex / len;
            const float cell = len / static_cast<float>(dim);
            const float range = first_pass ? fminf(fmaxf(1.15f * cell, 1.5f), 2.5f * cell)
                                           : fminf(fmaxf(0.30f * cell, 0.8f), 2.0f);
            const int half = min(max(2, static_cast<int>(ceilf(range / 0.75f))), kFitProbeHalf);
            const int probes = 2 * half + 1;
            const float step = range / static_cast<float>(half);
            const int samples = min(max(static_cast<int>(len / 6.0f), 8), 16);
            if (sample < samples) {
                const float alpha = static_cast<float>(sample + 1) / static_cast<float>(samples + 1);
                const float px = ax + alpha * ex;
                const float py = ay + alpha * ey;
                float best_mag = 0.0f;
                int best = -1;
                // One rise per probe, in order, with the reference's peak
                // scan.  (Blocks of four probes, the last block padded with
                // repeats of the last probe to keep loads in flight, issued
                // more instructions for the same result and ran slower.)
                for (int i = 0; i < probes; ++i) {
                    const float t = step * static_cast<float>(i - half);
                    const float m = rise_ro(image, width, height, stride, px + nx * t, py + ny * t, nx, ny);
                    mags[i] = m;
                    if (m > best_mag) {
                        best_mag = m;
                        best = i;
                    }
                }
                if (first_pass && best > 2) {
                    // The reference takes the first i in [1, best - 2] that is a local
                    // peak of at least 0.70 * best_mag with min(mags[i + 1 .. best - 1])
                    // below half of it.  One pass from the right with a running minimum
                    // finds the same i (the last one recorded) without the inner loop.
                    const float accept = 0.70f * best_mag;
                    float valley = FLT_MAX;
                    int first = -1;
                    for (int i = best - 2; i >= 1; --i) {
                        valley = fminf(valley, mags[i + 1]);
                        if (mags[i] < accept || mags[i] < mags[i - 1] || mags[i] < mags[i + 1]) continue;
                        if (valley < 0.5f * mags[i]) first = i;
                    }
                    if (first >= 0) {
                        best = first;
                        best_mag = mags[first];
                    }
                }
                if (best >= 0 && best_mag >= 6.0f) {
                    float t = step * static_cast<float>(best - half);
                    if (best > 0 && best < probes - 1) {
                        const float m0 = rise_ro(image, width, height, stride, px + nx * (t - step),
                                                 py + ny * (t - step), nx, ny);
                        const float m2 = rise_ro(image, width, height, stride, px + nx * (t + step),
                                                 py + ny * (t + step), nx, ny);
                        const float den = m0 - 2.0f * best_mag + m2;
                        if (den < -1e-3f) t += fminf(fmaxf(0.5f * (m0 - m2) / den, -0.5f), 0.5f) * step;
                    }
                    const float x = px + nx * t;
                    const float y = py + ny * t;
                    mx = x;
                    my = y;
                    mxx = x * x;
                    mxy = x * y;
                    myy = y * y;
                    used = 1;
                }
            }
        }
        // Levels of the reference tree that only add the zero lanes.
        for (int z = seg; z < 32; z <<= 1) {
            mx = mx + 0.0f;
            my = my + 0.0f;
            mxx = mxx + 0.0f;
            mxy = mxy + 0.0f;
            myy = myy + 0.0f;
        }
        for (int off = seg >> 1; off > 0; off >>= 1) {
            mx += __shfl_down_sync(kFull, mx, off, seg);
            my += __shfl_down_sync(kFull, my, off, seg);
            mxx += __shfl_down_sync(kFull, mxx, off, seg);
            mxy += __shfl_down_sync(kFull, mxy, off, seg);
            myy += __shfl_down_sync(kFull, myy, off, seg);
            used += __shfl_down_sync(kFull, used, off, seg);
        }
        if (sample == 0) {
            int ok = 0;
            if (edge_ok && used >= 4) {
                const float inv = 1.0f / static_cast<float>(used);
                const float cx = mx * inv;
                const float cy = my * inv;
                const float cxx = mxx * inv - cx * cx;
                const float cxy = mxy * inv - cx * cy;
                const float cyy = myy * inv - cy * cy;
                const float theta = 0.5f * bdmath::atan2(2.0f * cxy, cxx - cyy);
                float s, c;
                bdmath::sincos(theta, &s, &c);
                lines[edge][0] = cx;
                lines[edge][1] = cy;
                lines[edge][2] = -s;
                lines[edge][3] = c;
                ok = 1;
            }
            have[edge] = ok;
        }
    }
    __syncwarp();
}

// apply_refined_lines (reference :1021-1076) on lanes 0-3: lane i
// intersects lines i and i + 1 into corner i + 1; the maximum, the side
// checks and the signed area are then formed in the reference's order from
// the four lanes' values.  q (shared) is replaced by the refined quad when
// it is accepted; returns the largest corner move (0 when rejected).
__device__ float apply_refined_lines_warp(float (*q)[2], const float (*lines)[4], const int* have,
                                          int lane) {
    const int line_count = (have[0] ? 1 : 0) + (have[1] ? 1 : 0) + (have[2] ? 1 : 0) + (have[3] ? 1 : 0);
    if (line_count < 3) return 0.0f;
    const int i = lane & 3;
    const int j = (i + 1) & 3;
    const float qix = q[i][0], qiy = q[i][1];
    const float qjx = q[j][0], qjy = q[j][1];
    const float side = bdmath::hypot(qjx - qix, qjy - qiy);
    float extent = 0.0f;
    for (int k = 0; k < 4; ++k) extent = fmaxf(extent, __shfl_sync(kFull, side, k));
    const float max_shift = fminf(fmaxf(0.15f * extent, 4.0f), 16.0f);
    float rx = qjx, ry = qjy;  // refined corner j
    float shift = 0.0f;
    int shifted = 0;
    if (have[i] && have[j]) {
        float x, y;
        if (intersect_lines(lines[i], lines[j], &x, &y)) {
            const float dx = x - qjx;
            const float dy = y - qjy;
            if (!(dx * dx + dy * dy > max_shift * max_shift)) {
                rx = x;
                ry = y;
                shift = sqrtf(dx * dx + dy * dy);
                shifted = 1;
            }
        }
    }
    float moved = 0.0f;
    for (int k = 0; k < 4; ++k) {
        const float sk = __shfl_sync(kFull, shift, k);
        if (__shfl_sync(kFull, shifted, k)) moved = fmaxf(moved, sk);
    }
    // Refined corner i is held by lane (i + 3) & 3.
    const float pix = __shfl_sync(kFull, rx, (i + 3) & 3);
    const float piy = __shfl_sync(kFull, ry, (i + 3) & 3);
    const bool short_side = bdmath::hypot(rx - pix, ry - piy) < 3.0f;
    if (__any_sync(kFull, lane < 4 && short_side)) return 0.0f;
    const float term = pix * ry - rx * piy;
    float area2 = 0.0f;
    for (int k = 0; k < 4; ++k) area2 += __shfl_sync(kFull, term, k);
    if (area2 <= 0.0f) return 0.0f;
    __syncwarp();
    if (lane < 4) {
        q[j][0] = rx;
        q[j][1] = ry;
    }
    __syncwarp();
    return moved;
}

// One warp fits one edge for the CTA path of big candidates (reference
// fit_edge_line_warp :881-1016).  Sample s (< 16) along the edge is probed
// by lanes s and s + 16, which take the even and odd probe steps and leave
// the profile in shared memory; lane s then picks the peak exactly as the
// reference lane does.  The moments sit in lanes 0..15 (zero above), so the
// shuffle tree sums them in the reference's order.
__device__ bool fit_edge_line_warp(const float quad[4][2], int edge, const uint8_t* __restrict__ image,
                                   int width, int height, int64_t stride, int dim, bool first_pass,
                                   int lane, float* s_mags, float line[4]) {
    const int bi = (edge + 1) & 3;
    const float ax = quad[edge][0], ay = quad[edge][1];
    const float bx = quad[bi][0], by = quad[bi][1];
    const float ex = bx - ax;
    const float ey = by - ay;
    const float len = sqrtf(ex * ex + ey * ey);
    if (len < 8.0f) return false;
    const float nx = ey / len;
    const float ny = -ex / len;
    const float cell = len / static_cast<float>(dim);
    const float range = first_pass ? fminf(fmaxf(1.15f * cell, 1.5f), 2.5f * cell)
                                   : fminf(fmaxf(0.30f * cell, 0.8f), 2.0f);
    const int half = min(max(2, static_cast<int>(ceilf(range / 0.75f))), kFitProbeHalf);
    const int probes = 2 * half + 1;
    const float step = range / static_cast<float>(half);
    const int samples = min(max(static_cast<int>(len / 6.0f), 8), 16);

    const int sample = lane & 15;
    const int parity = lane >> 4;
    float px = 0.0f, py = 0.0f;
    if (sample < samples) {
        const float alpha = static_cast<float>(sample + 1) / static_cast<float>(samples + 1);
        px = ax + alpha * ex;
        py = ay + alpha * ey;
        float* mags = s_mags + sample * kMaxProbes;
#pragma unroll 1
        for (int i = parity; i < probes; i += 2) {
            const float t = step * static_cast<float>(i - half);
            mags[i] = rise_ro(image, width, height, stride, px + nx * t, py + ny * t, nx, ny);
        }
    }
    __syncwarp();

    float mx = 0.0f, my = 0.0f, mxx = 0.0f, mxy = 0.0f, myy = 0.0f;
    int used = 0;
    if (parity == 0 && sample < samples) {
        const float* mags = s_mags + sample * kMaxProbes;
        float best_mag = 0.0f;
        int best = -1;
        for (int i = 0; i < probes; ++i) {
            const float mag = mags[i];
            if (mag > best_mag) {
                best_mag = mag;
                best = i;
            }
        }
        if (first_pass && best > 2) {
            // The reference takes the first i in [1, best - 2] that is a local
            // peak of at least 0.70 * best_mag with min(mags[i + 1 .. best - 1])
            // below half of it.  One pass from the right with a running minimum
            // finds the same i (the last one recorded) without the inner loop.
            const float accept = 0.70f * best_mag;
            float valley = FLT_MAX;
            int first = -1;
            for (int i = best - 2; i >= 1; --i) {
                valley = fminf(valley, mags[i + 1]);
                if (mags[i] < accept || mags[i] < mags[i - 1] || mags[i] < mags[i + 1]) continue;
                if (valley < 0.5f * mags[i]) first = i;
            }
            if (first >= 0) {
                best = first;
                best_mag = mags[first];
            }
        }
        if (best >= 0 && best_mag >= 6.0f) {
            float t = step * static_cast<float>(best - half);
            if (best > 0 && best < probes - 1) {
                const float m0 = rise_ro(image, width, height, stride, px + nx * (t - step),
                                         py + ny * (t - step), nx, ny);
                const float m2 = rise_ro(image, width, height, stride, px + nx * (t + step),
                                         py + ny * (t + step), nx, ny);
                const float den = m0 - 2.0f * best_mag + m2;
                if (den < -1e-3f) t += fminf(fmaxf(0.5f * (m0 - m2) / den, -0.5f), 0.5f) * step;
            }
            const float x = px + nx * t;
            const float y = py + ny * t;
            mx = x;
            my = y;
            mxx = x * x;
            mxy = x * y;
            myy = y * y;
            used = 1;
        }
    }
    for (int off = 16; off > 0; off >>= 1) {
        mx += __shfl_down_sync(kFull, mx, off);
        my += __shfl_down_sync(kFull, my, off);
        mxx += __shfl_down_sync(kFull, mxx, off);
        mxy += __shfl_down_sync(kFull, mxy, off);
        myy += __shfl_down_sync(kFull, myy, off);
        used += __shfl_down_sync(kFull, used, off);
    }
    __syncwarp();
    if (lane != 0) return true;
    if (used < 4) return false;
    const float inv = 1.0f / static_cast<float>(used);
    const float cx = mx * inv;
    const float cy = my * inv;
    const float cxx = mxx * inv - cx * cx;
    const float cxy = mxy * inv - cx * cy;
    const float cyy = myy * inv - cy * cy;
    const float theta = 0.5f * bdmath::atan2(2.0f * cxy, cxx - cyy);
    float s, c;
    bdmath::sincos(theta, &s, &c);
    line[0] = cx;
    line[1] = cy;
    line[2] = -s;
    line[3] = c;
    return true;
}

// ---- decode of one variant (reference homography_from_unit_quad :1249,
// match_code :1274, decode_quad :1291) ----
__device__ __forceinline__ bool homography_from_unit_quad(const float quad[4][2], float h[9]) {
    const float x0 = quad[0][0], y0 = quad[0][1];
    const float x1 = quad[1][0], y1 = quad[1][1];
    const float x2 = quad[2][0], y2 = quad[2][1];
    const float x3 = quad[3][0], y3 = quad[3][1];
    const float dx1 = x1 - x2, dx2 = x3 - x2, dx3 = x0 - x1 + x2 - x3;
    const float dy1 = y1 - y2, dy2 = y3 - y2, dy3 = y0 - y1 + y2 - y3;
    const float det = dx1 * dy2 - dx2 * dy1;
    if (fabsf(det) < 1e-9f) return false;
    const float g = (dx3 * dy2 - dx2 * dy3) / det;
    const float k = (dx1 * dy3 - dx3 * dy1) / det;
    h[0] = x1 - x0 + g * x1;
    h[1] = x3 - x0 + k * x3;
    h[2] = x0;
    h[3] = y1 - y0 + g * y1;
    h[4] = y3 - y0 + k * y3;
    h[5] = y0;
    h[6] = g;
    h[7] = k;
    h[8] = 1.0f;
    return true;
}

struct VariantResult {
    int id;
    int hamming;
    float margin;
    float corners[8];
};

// c / dim for a cell index c < 64 of a 6- or 8-cell grid without an
// integer division: (c * 43) >> 8 == c / 6 for every c < 128.
__device__ __forceinline__ int cell_row(int c, int dim) { return dim == 8 ? (c >> 3) : ((c * 43) >> 8); }

// Decodes the four rotations of one quad at once (reference decode_quad
// :1291-1436, one call per variant there): lanes 8r..8r+7 take rotation r,
// lane 8r+u sampling cells u, u+8, ... of the dim x dim grid with the
// reference's expressions (cell centres (c + 0.5f) / dim from cell_uv, the
// same divisions done once per CTA).  Per rotation, the valid flag, min/max, border
// test and code bits are reduced inside the 8-lane group (all, min, max and
// OR do not depend on order).  Every lane then scores codewords i = lane,
// lane+32, ... against all four codes (the first codeword at the minimum
// distance, as match_code :1274), and each group leader forms the decision
// margin with the reference's row-major sums.  Returns, in all lanes, the
// rotation with the highest score (4 - hamming) * 1000 + margin, the first
// on ties, or -1; lane 0 writes its record to *result.
__device__ int decode_rotations_warp(const uint8_t* __restrict__ gray, const FrameDesc& d,
                                     int64_t stride, int fam, const float* src, int lane,
                                     const float* cell_uv, float (*s_raw)[64], float (*s_sharp)[64],
                                     VariantResult* result) {
    const int dim = family_dim(fam);
    const int cells = dim * dim;
    const int g = lane >> 3;
    const int u = lane & 7;
    const uint32_t gmask = 0xffu << (8 * g);
    float corners[4][2];
    for (int k = 0; k < 4; ++k) {
        const int s = (g + k) & 3;
        corners[k][0] = src[s * 2 + 0];
        corners[k][1] = src[s * 2 + 1];
    }
    float h[9];
    bool alive = homography_from_unit_quad(corners, h);
    bool valid = true;
    float mn = 255.0f, mx = 0.0f;
    float* raw = s_raw[g];
    if (alive) {
        for (int c = u; c < cells; c += 8) {
            const int cy = cell_row(c, dim), cx = c - cy * dim;
            const float uu = cell_uv[cx];  // (cx + 0.5f) / dim
            const float vv = cell_uv[cy];
            const float den = h[6] * uu + h[7] * vv + 1.0f;
            if (fabsf(den) < 1e-9f) {
                valid = false;
                continue;
            }
            const float x = (h[0] * uu + h[1] * vv + h[2]) / den;
            const float y = (h[3] * uu + h[4] * vv + h[5]) / den;
            const float value = sample_ro(gray, d.width, d.height, stride, x - 0.0f, y - 0.0f);
            if (value < 0.0f) valid = false;
            raw[c] = value;
            mn = fminf(mn, value);
            mx = fmaxf(mx, value);
        }
    }
    valid = (__ballot_sync(kFull, valid) & gmask) == gmask;
    for (int off = 4; off > 0; off >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(kFull, mn, off));
        mx = fmaxf(mx, __shfl_xor_sync(kFull, mx, off));
    }
    alive = alive && valid && !(mx - mn < 10.0f);
    const float thresh = 0.5f * (mn + mx);
    bool border_bad = false;
    if (alive) {
        for (int c = u; c < cells; c += 8) {
            const int cy = cell_row(c, dim), cx = c - cy * dim;
            if (cx == 0 || cy == 0 || cx == dim - 1 || cy == dim - 1) {
                border_bad = border_bad || raw[c] >= thresh;
            }
        }
    }
    alive = alive && (__ballot_sync(kFull, border_bad) & gmask) == 0;
    __syncwarp();
    if (alive) {
        for (int c = u; c < cells; c += 8) raw[c] = raw[c] - thresh;  // diff
    }
    __syncwarp();
    const int nbits = (dim - 2) * (dim - 2);
    uint64_t code_part = 0;
    if (alive) {
        float* sharp = s_sharp[g];
        for (int c = u; c < cells; c += 8) {
            const int cy = cell_row(c, dim), cx = c - cy * dim;
            float sv = raw[c];
            if (cx >= 1 && cy >= 1 && cx <= dim - 2 && cy <= dim - 2) {
                const float cc = raw[c];
                const float lap = 4.0f * cc - raw[c - dim] - raw[c + dim] - raw[c - 1] - raw[c + 1];
                sv = cc + d.sharpening * lap;
                const int k = (cy - 1) * (dim - 2) + (cx - 1);
                if (sv > 0.0f) code_part |= 1ull << (nbits - 1 - k);
            }
            sharp[c] = sv;
        }
    }
    for (int off = 4; off > 0; off >>= 1) code_part |= __shfl_xor_sync(kFull, code_part, off);
    const uint32_t alive_lanes = __ballot_sync(kFull, alive);
    if (alive_lanes == 0) return -1;

    // Codeword search for the four codes together.
    const uint64_t* codes = fam == 0 ? d_codes36h11 : d_codes16h5;
    const int code_count = fam == 0 ? BD_CODEWORDS_36H11_COUNT : BD_CODEWORDS_16H5_COUNT;
    uint64_t code[4];
    uint32_t key[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        code[r] = __shfl_sync(kFull, code_part, 8 * r);
        key[r] = 0xffffffffu;
    }
    for (int i = lane; i < code_count; i += 32) {
        const uint64_t cw = codes[i];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t dist = static_cast<uint32_t>(__popcll(cw ^ code[r]));
            key[r] = min(key[r], (dist << 16) | static_cast<uint32_t>(i));
        }
    }
    uint32_t my_key = 0xffffffffu;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const uint32_t k = __reduce_min_sync(kFull, key[r]);
        if (g == r) my_key = k;
    }
    const int best_dist = static_cast<int>(my_key >> 16);
    alive = alive && best_dist <= d.max_hamming[fam];
    __syncwarp();
    // Decision margin on the group leader: sums in row-major order of the
    // data cells.
    float margin = 0.0f;
    if (alive && u == 0) {
        const float* sharp = s_sharp[g];
        float white_sum = 0.0f, black_sum = 0.0f;
        int white_count = 0, black_count = 0;
        for (int cy = 1; cy <= dim - 2; ++cy) {
            for (int cx = 1; cx <= dim - 2; ++cx) {
                const float dv = sharp[cy * dim + cx];
                if (dv > 0.0f) {
                    white_sum += dv;
                    ++white_count;
                } else {
                    black_sum -= dv;
                    ++black_count;
                }
            }
        }
        const float white_avg = white_sum / static_cast<float>(max(white_count, 1));
        const float black_avg = black_sum / static_cast<float>(max(black_count, 1));
        margin = fminf(white_avg, black_avg);
        alive = !(margin < d.min_margin);
    }
    // Best rotation, first on ties (reference k_decode_quads :1448-1460).
    int best = -1;
    float best_score = -1.0f;
    float best_margin = 0.0f;
    uint32_t best_key = 0;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const bool ok = __shfl_sync(kFull, alive ? 1 : 0, 8 * r) != 0;
        const float m = __shfl_sync(kFull, margin, 8 * r);
        const uint32_t k = __shfl_sync(kFull, my_key, 8 * r);
        if (!ok) continue;
        const float score = static_cast<float>(4 - static_cast<int>(k >> 16)) * 1000.0f + m;
        if (score > best_score) {
            best_score = score;
            best = r;
            best_margin = m;
            best_key = k;
        }
    }
    if (best >= 0 && lane == 0) {
        result->id = static_cast<int>(best_key & 0xffffu);
        result->hamming = static_cast<int>(best_key >> 16);
        result->margin = best_margin;
        for (int k = 0; k < 4; ++k) {
            const int s = (best + k) & 3;
            result->corners[k * 2 + 0] = src[s * 2 + 0];
            result->corners[k * 2 + 1] = src[s * 2 + 1];
        }
    }
    __syncwarp();
    return best;
}

// ===========================================================================
// 7+8. Quad fit and decode, one warp per candidate (reference k_fit_quads
//    :1081-1241 with helpers :659-1076, and k_decode_quads :1438 with
//    homography_from_unit_quad :1249, match_code :1274, decode_quad :1291).
//    The warp builds the hull and its four-corner quad, then for each
//    requested family refines the quad's edges and decodes it: rotations
//    0-3 of the refined quad, and rotations 0-3 of the hull quad only when
//    none of those decoded (the reference's variant order and score).
// ===========================================================================

// Per-warp shared memory of k_fit_decode.
struct QuadSmem {
    // The probe profiles live only while edges are refined, the decode
    // cells only while the quad is decoded: they share the space.
    union {
        float mags[32 * kMaxProbes];  // one probe profile per lane
        struct {
            float raw[4][64];         // per rotation: samples, then differences
            float sharp[4][64];
        } cells;
    };
    uint32_t hull[32];
    float q[4][2];                // quad being refined
    float hq[4][2];               // hull quad
    float lines[4][4];
    int have[4];
    VariantResult res;
};

// Leftmost / rightmost run of component `root` in row y within [x0, x1]
// (reference collect_row_extremes :676-715): binary search for the first
// run ending at or after x0, then runs in order until one starts past x1.
__device__ __forceinline__ void row_extremes(const FrameDesc& d, uint32_t root, int x0, int x1, int y,
                                             uint32_t* left_point, uint32_t* right_point) {
    const int n = static_cast<int>(d.row_count[y]);
    const uint32_t* row_runs = d.runs + static_cast<int64_t>(y) * d.row_cap;
    const uint32_t* row_label = d.parent + static_cast<int64_t>(y) * d.row_cap;
    // First run ending at or after x0 (runs of a row are sorted): eight-way
    // steps of seven independent loads, then the last <= 8 runs at once.
    int lo = 0, hi = n;  // the answer lies in [lo, hi]; hi = n: none
    while (hi - lo > 8) {
        const int span = hi - lo;
        uint32_t v[7];
#pragma unroll
        for (int k = 0; k < 7; ++k) v[k] = row_runs[lo + (span * (k + 1)) / 8];
        int nlo = lo, nhi = hi;
#pragma unroll
        for (int k = 6; k >= 0; --k) {
            const int idx = lo + (span * (k + 1)) / 8;
            if (static_cast<int>(v[k] >> 16) >= x0) nhi = idx; else if (nlo == lo) nlo = idx + 1;
        }
        lo = nlo;
        hi = nhi;
    }
    int first = hi;
    {
        uint32_t v[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = row_runs[min(lo + k, max(n - 1, 0))];
#pragma unroll
        for (int k = 7; k >= 0; --k) {
            if (lo + k < hi && static_cast<int>(v[k] >> 16) >= x0) first = lo + k;
        }
    }
    int left = -1, right = -1;
    // Runs two at a time (no padding loads past the end of the row).
    for (int k = first; k < n; k += 2) {
        uint32_t rr[2] = {}, lab[2] = {};
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (k + j < n) {
                rr[j] = row_runs[k + j];
                lab[j] = row_label[k + j];
            }
        }
        bool stop = false;
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            if (stop || k + j >= n) continue;
            const int rx0 = static_cast<int>(rr[j] & 0xffffu);
            const int rx1 = static_cast<int>(rr[j] >> 16);
            if (rx0 > x1) {
                stop = true;
                continue;
            }
            if (lab[j] != root) continue;
            left = left < 0 ? rx0 : min(left, rx0);
            right = right < 0 ? rx1 : max(right, rx1);
        }
        if (stop) break;
    }
    *left_point = left < 0 ? kNone : pack_point(left, y);
    *right_point = right < 0 ? kNone : pack_point(right, y);
}

// Refinement and decode of one (candidate, family) item by one warp, from
// the hull quad in sm.hq / sm.q.
__device__ void fit_decode_family(const FrameDesc& d, int fam, int ci, const uint8_t* __restrict__ gray,
                                  int64_t stride, bool quad_ok, int lane, const float* cell_uv,
                                  QuadSmem& sm) {
    const int mc = d.max_candidates;
    {
        float* quad_out = d.quads + (static_cast<int64_t>(fam) * mc + ci) * 8;
        DecodeOut* out = d.decodes + static_cast<int64_t>(fam) * mc + ci;
        if (!quad_ok) {
            if (lane < 8) quad_out[lane] = bdmath::quiet_nan();
            if (lane == 0) out->id = -1;
            __syncwarp();
            return;
        }
        const int dim = family_dim(fam);
        for (int iteration = 0; d.refine_edges && iteration < kFitIterations; ++iteration) {
            fit_edges_warp(sm.q, gray, d.width, d.height, stride, dim, iteration == 0, lane, sm.mags,
                           sm.lines, sm.have);
            const float moved = apply_refined_lines_warp(sm.q, sm.lines, sm.have, lane);
            // Converged quads skip the second pass (reference :1229-1231).
            if (moved < 0.15f) break;
        }
        if (lane < 8) quad_out[lane] = sm.q[lane >> 1][lane & 1];

        // Decode: the refined quad's rotations, then the hull quad's only
        // when none of those decoded and refinement moved a corner (an
        // unmoved quad would decode the same way again).  One call site in
        // a loop that is not unrolled keeps one copy of the decode code.
        bool moved = false;
        {
            const float* qa = &sm.q[0][0];
            const float* qb = &sm.hq[0][0];
            for (int k = 0; k < 8; ++k) moved = moved || __float_as_uint(qa[k]) != __float_as_uint(qb[k]);
        }
        int best = -1;
#pragma unroll 1
        for (int variant = 0; variant < 2; ++variant) {
            if (variant == 1 && (best >= 0 || !moved)) break;
            best = decode_rotations_warp(gray, d, stride, fam, variant == 0 ? &sm.q[0][0] : &sm.hq[0][0], lane,
                                         cell_uv, sm.cells.raw, sm.cells.sharp, &sm.res);
        }
        if (lane == 0) {
            if (best < 0) {
                out->id = -1;
            } else {
                out->id = sm.res.id;
                out->hamming = sm.res.hamming;
                out->margin = sm.res.margin;
                for (int k = 0; k < 8; ++k) out->corners[k] = sm.res.corners[k];
            }
        }
        __syncwarp();
    }
}


// One (small candidate, family) item by one warp: candidate k of the back
// of the frame's fit list, family slot `slot` (0: the lowest requested
// family).  The warp builds the candidate's hull itself (slot 0 also stores
// it), so the families of a candidate proceed concurrently and warps never
// wait for one another.  (ux, uy): this lane's probe direction; uv: cell
// centres per family.
__device__ __forceinline__ void fit_small_item(const BatchDesc* __restrict__ b,
                                               const FrameIO* __restrict__ io, int fi, int k, int slot,
                                               float ux, float uy, const float (*uv)[8], QuadSmem& sm,
                                               int lane) {
    const FrameDesc& d = b->f[fi];
    const uint32_t fams = d.families & 3u;
    const int ci = static_cast<int>(d.fit_list[d.max_candidates - 1 - k]);
    const int fam = (slot == 0 && (fams & 1u)) ? 0 : 1;
    const bool first_family = slot == 0;
    const uint8_t* __restrict__ gray = io[fi].gray;
    const int64_t stride = io[fi].stride;
    const uint32_t root = d.candidates[ci];
    const uint4 bb = reinterpret_cast<const uint4*>(d.bbox)[root];
    const int x0 = static_cast<int>(bb.x), y0 = static_cast<int>(bb.y);
    const int x1 = static_cast<int>(bb.z), y1 = static_cast<int>(bb.w);
    const int rows = y1 - y0 + 1;
    const int kept = min(rows, kMaxBoundaryRows);

    // Boundary points in reference order (row s: left, then right) go
    // to every lane by shuffles; lane = direction keeps the first point
    // of largest projection.  The points travel as float coordinates,
    // converted once by the lane that found them (NaN for a row without a
    // point: its projection never wins), and the winning point's packed
    // form is fetched once per round.
    float best_dot = -FLT_MAX;
    uint32_t best_point = kNone;
    const float none = bdmath::quiet_nan();
    for (int s0 = 0; s0 < kept; s0 += 32) {
        uint32_t lp = kNone, rp = kNone;
        const int s = s0 + lane;
        if (s < kept) {
            const int y = y0 + (kept == rows ? s : (s * (rows - 1)) / (kept - 1));  // kept < rows: kept > 1
            row_extremes(d, root, x0, x1, y, &lp, &rp);
        }
        const float lx = lp != kNone ? static_cast<float>(lp & 0xffffu) : none;
        const float ly = lp != kNone ? static_cast<float>(lp >> 16) : none;
        const float rx = rp != kNone ? static_cast<float>(rp & 0xffffu) : none;
        const float ry = rp != kNone ? static_cast<float>(rp >> 16) : none;
        const int count = min(32, kept - s0);
        int pick = -1;  // 2 * row + side of this round's best point
        for (int k = 0; k < count; ++k) {
            const float ax = __shfl_sync(kFull, lx, k), ay = __shfl_sync(kFull, ly, k);
            const float bx = __shfl_sync(kFull, rx, k), by = __shfl_sync(kFull, ry, k);
            const float dl = ax * ux + ay * uy;
            if (dl > best_dot) {
                best_dot = dl;
                pick = 2 * k;
            }
            const float dr = bx * ux + by * uy;
            if (dr > best_dot) {
                best_dot = dr;
                pick = 2 * k + 1;
            }
        }
        const uint32_t cl = __shfl_sync(kFull, lp, max(pick, 0) >> 1);
        const uint32_t cr = __shfl_sync(kFull, rp, max(pick, 0) >> 1);
        if (pick >= 0) best_point = (pick & 1) ? cr : cl;
    }
    // Hull: extremes in direction order without repeats of the previous
    // kept point, and without a last point equal to the first.  The
    // previous kept point equals the nearest earlier valid extreme.
    const bool valid = best_point != kNone;
    const uint32_t vmask = __ballot_sync(kFull, valid);
    const uint32_t earlier = vmask & lanemask_lt();
    const int prev_lane = earlier ? 31 - __clz(earlier) : 0;
    const uint32_t prev_point = __shfl_sync(kFull, best_point, prev_lane);
    const bool keep = valid && (earlier == 0 || prev_point != best_point);
    const uint32_t kmask = __ballot_sync(kFull, keep);
    if (keep) sm.hull[__popc(kmask & lanemask_lt())] = best_point;
    __syncwarp();
    int hc = __popc(kmask);
    while (hc > 1 && sm.hull[0] == sm.hull[hc - 1]) --hc;

    float quad[4][2] = {};
    const bool quad_ok = hull_to_quad_warp(sm.hull, hc, quad, lane);
    {
        float v = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) v = lane == k ? quad[k >> 1][k & 1] : v;
        if (lane < 8) {
            sm.hq[lane >> 1][lane & 1] = v;
            sm.q[lane >> 1][lane & 1] = v;
            if (first_family) {
                d.hull_quads[static_cast<int64_t>(ci) * 8 + lane] = quad_ok ? v : bdmath::quiet_nan();
            }
        }
    }
    if (lane == 0 && quad_ok && first_family) atomicAdd(&d.state->counts[3], 1u);
    __syncwarp();
    fit_decode_family(d, fam, ci, gray, stride, quad_ok, lane, uv[fam], sm);
}

// Shared memory of fit_big_item.
struct BigSmem {
    uint32_t boundary[2 * kMaxBoundaryRows];
    float probe_dot[8][kFitDirections];
    uint32_t probe_point[8][kFitDirections];
    uint32_t s_hull[kFitDirections];
    float hull_quad[4][2];
    float fit_quad[2][4][2];
    float edge_lines[2][4][4];
    int edge_have[2][4];
    int quad_ok;
    int s_done[2];
    float s_mags[8][16 * kMaxProbes];
    float s_raw[4][4][64];
    float s_sharp[4][4][64];
    VariantResult s_res[4];
    int s_best[4];
};

// One big candidate by a whole CTA of 8 warps: candidate k of the front of
// frame fi's fit list.  The boundary rows are spread over 256 threads, every
// warp takes a slice of the boundary for the 32 probe directions, warp 0
// builds the hull and its quad, warps 4s..4s+3 refine the quad of family
// slot s (one warp per edge), and warps 2s / 2s+1 decode the refined / hull
// quad of slot s (the hull result is used only when no refined rotation
// decodes).
__device__ __forceinline__ void fit_big_item(const BatchDesc* __restrict__ b,
                                             const FrameIO* __restrict__ io, int fi, int k, float ux,
                                             float uy, const float (*s_uv)[8], BigSmem& sm) {
    constexpr int kWarps = 8;
    const int tid = threadIdx.x;
    const int warp = tid >> 5, lane = tid & 31;
    const FrameDesc& d = b->f[fi];
    const int ci = static_cast<int>(d.fit_list[k]);
    const int mc = d.max_candidates;
    const uint8_t* __restrict__ gray = io[fi].gray;
    const int64_t stride = io[fi].stride;
    const uint32_t root = d.candidates[ci];
    const uint4 bb = reinterpret_cast<const uint4*>(d.bbox)[root];
    const int x0 = static_cast<int>(bb.x), y0 = static_cast<int>(bb.y);
    const int x1 = static_cast<int>(bb.z), y1 = static_cast<int>(bb.w);
    const int rows = y1 - y0 + 1;
    const int kept = min(rows, kMaxBoundaryRows);
    const int points = 2 * kept;

    for (int s = tid; s < kept; s += blockDim.x) {
        const int y = y0 + (kept == rows ? s : (s * (rows - 1)) / (kept - 1));  // kept < rows: kept > 1
        row_extremes(d, root, x0, x1, y, &sm.boundary[2 * s], &sm.boundary[2 * s + 1]);
    }
    __syncthreads();
    // Extreme point per direction over this warp's slice; slices
    // are merged in order, so the first point still wins ties.
    {
        const int slice = (points + kWarps - 1) / kWarps;
        const int begin = warp * slice;
        const int end = min(points, begin + slice);
        float best_dot = -FLT_MAX;
        uint32_t best_point = kNone;
        for (int i = begin; i < end; ++i) {
            const uint32_t p = sm.boundary[i];
            if (p == kNone) continue;
            const float dd =
                static_cast<float>(p & 0xffffu) * ux + static_cast<float>(p >> 16) * uy;
            if (dd > best_dot) {
                best_dot = dd;
                best_point = p;
            }
        }
        sm.probe_dot[warp][lane] = best_dot;
        sm.probe_point[warp][lane] = best_point;
    }
    __syncthreads();
    if (warp == 0) {
        float best_dot = -FLT_MAX;
        uint32_t best_point = kNone;
        for (int p = 0; p < kWarps; ++p) {
            if (sm.probe_dot[p][lane] > best_dot) {
                best_dot = sm.probe_dot[p][lane];
                best_point = sm.probe_point[p][lane];
            }
        }
        const bool valid = best_point != kNone;
        const uint32_t vmask = __ballot_sync(kFull, valid);
        const uint32_t earlier = vmask & lanemask_lt();
        const int prev_lane = earlier ? 31 - __clz(earlier) : 0;
        const uint32_t prev_point = __shfl_sync(kFull, best_point, prev_lane);
        const bool keep = valid && (earlier == 0 || prev_point != best_point);
        const uint32_t kmask = __ballot_sync(kFull, keep);
        if (keep) sm.s_hull[__popc(kmask & lanemask_lt())] = best_point;
        __syncwarp();
        int hc = __popc(kmask);
        while (hc > 1 && sm.s_hull[0] == sm.s_hull[hc - 1]) --hc;
        float quad[4][2] = {};
        const bool ok = hull_to_quad_warp(sm.s_hull, hc, quad, lane);
        float v = 0.0f;
#pragma unroll
        for (int k = 0; k < 8; ++k) v = lane == k ? quad[k >> 1][k & 1] : v;
        if (lane < 8) {
            sm.hull_quad[lane >> 1][lane & 1] = v;
            sm.fit_quad[0][lane >> 1][lane & 1] = v;
            sm.fit_quad[1][lane >> 1][lane & 1] = v;
            d.hull_quads[static_cast<int64_t>(ci) * 8 + lane] = ok ? v : bdmath::quiet_nan();
        }
        if (lane == 0) {
            sm.quad_ok = ok ? 1 : 0;
            if (ok) atomicAdd(&d.state->counts[3], 1u);
        }
    }
    __syncthreads();

    const uint32_t fams = d.families & 3u;
    const int nfam = __popc(fams);
    const int fam_of_slot[2] = {(fams & 1u) ? 0 : 1, 1};
    if (!sm.quad_ok) {
        if (tid < 8 * nfam) {
            const int fam = fam_of_slot[tid >> 3];
            d.quads[(static_cast<int64_t>(fam) * mc + ci) * 8 + (tid & 7)] = bdmath::quiet_nan();
        }
        if (tid < nfam) d.decodes[static_cast<int64_t>(fam_of_slot[tid]) * mc + ci].id = -1;
        __syncthreads();
        return;
    }
    if (d.refine_edges) {
        const int slot = warp >> 2;
        const int edge = warp & 3;
        const bool mine = slot < nfam;
        const int dim = family_dim(fam_of_slot[mine ? slot : 0]);
        if (tid < 2) sm.s_done[tid] = 0;
        __syncthreads();
        for (int iteration = 0; iteration < kFitIterations; ++iteration) {
            if (mine && !sm.s_done[slot]) {
                float line[4];
                const bool ok = fit_edge_line_warp(sm.fit_quad[slot], edge, gray, d.width, d.height,
                                                   stride, dim, iteration == 0, lane, sm.s_mags[warp],
                                                   line);
                if (lane == 0) {
                    sm.edge_have[slot][edge] = ok ? 1 : 0;
                    if (ok) {
                        for (int k = 0; k < 4; ++k) sm.edge_lines[slot][edge][k] = line[k];
                    }
                }
            }
            __syncthreads();
            if (edge == 0 && mine && !sm.s_done[slot]) {
                const float moved =
                    apply_refined_lines_warp(sm.fit_quad[slot], sm.edge_lines[slot], sm.edge_have[slot], lane);
                // Converged quads skip the second pass (reference :1229-1231).
                if (lane == 0 && moved < 0.15f) sm.s_done[slot] = 1;
            }
            __syncthreads();
        }
    }
    if (tid < 8 * nfam) {
        const int slot = tid >> 3;
        const int fam = fam_of_slot[slot];
        d.quads[(static_cast<int64_t>(fam) * mc + ci) * 8 + (tid & 7)] =
            sm.fit_quad[slot][(tid & 7) >> 1][tid & 1];
    }
    bool hull_needed = false;  // refinement moved a corner of this warp's slot
    if (warp < 2 * nfam) {
        const float* qa = &sm.fit_quad[warp >> 1][0][0];
        const float* qb = &sm.hull_quad[0][0];
        for (int k = 0; k < 8; ++k) {
            hull_needed = hull_needed || __float_as_uint(qa[k]) != __float_as_uint(qb[k]);
        }
    }
    if (warp < 2 * nfam && ((warp & 1) == 0 || hull_needed)) {
        const int slot = warp >> 1;
        const float* src = (warp & 1) == 0 ? &sm.fit_quad[slot][0][0] : &sm.hull_quad[0][0];
        const int best = decode_rotations_warp(gray, d, stride, fam_of_slot[slot], src, lane,
                                               s_uv[fam_of_slot[slot]], sm.s_raw[warp],
                                               sm.s_sharp[warp], &sm.s_res[warp]);
        if (lane == 0) sm.s_best[warp] = best;
    } else if (warp < 2 * nfam && lane == 0) {
        sm.s_best[warp] = -1;  // unmoved quad: the refined decode covers it
    }
    __syncthreads();
    if (tid < nfam) {
        DecodeOut* out = d.decodes + static_cast<int64_t>(fam_of_slot[tid]) * mc + ci;
        const int pick = sm.s_best[2 * tid] >= 0 ? 2 * tid : (sm.s_best[2 * tid + 1] >= 0 ? 2 * tid + 1 : -1);
        if (pick < 0) {
            out->id = -1;
        } else {
            out->id = sm.s_res[pick].id;
            out->hamming = sm.s_res[pick].hamming;
            out->margin = sm.s_res[pick].margin;
            for (int k = 0; k < 8; ++k) out->corners[k] = sm.s_res[pick].corners[k];
        }
    }
    __syncthreads();
}

}  // namespace
}  // namespace bdgb
