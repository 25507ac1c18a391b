// Stages 1-5 of the pipeline as device functions of one CTA and one unit of
// work (a frame's tile rows or band): tile statistics, binarization with
// band-local components, boundary unions, root aggregates, candidate
// selection and ordering.  The per-stage kernels (k_front.cu) and the
// persistent kernel (k_persistent.cu) both call them.  Every function
// expects blockDim.x == 256 and takes its shared memory as a struct, so a
// persistent kernel can overlay the stages' shared memory.  All FP32
// arithmetic follows the reference expressions term by term and is compiled
// with -fmad=false.
#pragma once

#include "kernels_common.cuh"
#include "kernels.cuh"

namespace bdgb {
namespace {

constexpr int kMaxStatsRowsPerCta = 4;

struct StatsSmem {
    uint32_t span[256];
    uint32_t mean[64];
    int lo[kMaxStatsRowsPerCta], hi[kMaxStatsRowsPerCta];
};

// Static part of stage_binarize's shared memory; the run arrays and bit rows
// (band_smem_bytes) are a separate dynamic region.
struct BinSmem {
    RefSmem ref;
    uint32_t refs[2];          // the frame references (span quartile, Otsu level)
    uint8_t thresh[BD_MAX_WIDTH / kTile];
    uint8_t vmin[BD_MAX_WIDTH / kTile];
    uint8_t vmax[BD_MAX_WIDTH / kTile];
    uint32_t rowtot[kTile];
    uint32_t rowoff[kTile + 1];
    uint32_t nroots;
    uint32_t segmask;
};

// stage_cand's shared memory, besides the per-band candidate prefix (tile_h
// + 1 words of the tallest frame, a separate region).
struct CandSmem {
    uint32_t rowoff[kTile + 1];
    uint32_t wbin[8][64];
    uint32_t run[64];
    uint32_t chunk[4][64];
    uint32_t total[64];
    uint32_t base[64];
    uint32_t warp_sum[8];
    uint32_t ncand, limit, nbig, nsmall;
    int last;
};

// ===========================================================================
// 1. Tile statistics, histograms and active extents.  The frame references
//    that the histograms give are computed where they are used, by every
//    band of stage 2 (the reference's k_tile_reference :174-230 is a single
//    thread between the two).  CTA `cta` of frame fi covers
//    `stats_rows` tile rows; thread i of the CTA takes tile pair i (two
//    horizontally adjacent tiles, 128-bit loads), row-major over those rows.
// ===========================================================================
__device__ __forceinline__ void stage_stats(const BatchDesc* __restrict__ b, const FrameIO* __restrict__ io, int fi,
                            int cta, StatsSmem& sm) {
    uint32_t* s_span = sm.span;
    uint32_t* s_mean = sm.mean;
    int* s_lo = sm.lo;
    int* s_hi = sm.hi;
    const int tid = threadIdx.x;
    const FrameDesc& d = b->f[fi];
    FrameState* st = d.state;
    const int ty0 = cta * b->stats_rows;
    const int nrows = min(b->stats_rows, d.tile_h - ty0);

    s_span[tid] = 0;
    if (tid < 64) s_mean[tid] = 0;
    if (tid < kMaxStatsRowsPerCta) {
        s_lo[tid] = INT_MAX;
        s_hi[tid] = -1;
    }
    __syncthreads();

    const uint8_t* gray = io[fi].gray;
    const int64_t stride = io[fi].stride;
    const int W = d.width, H = d.height, tw = d.tile_w;
    const bool vec16 = ((reinterpret_cast<uintptr_t>(gray) | static_cast<uintptr_t>(stride)) & 15u) == 0;
    const int pairs = (tw + 1) >> 1;
    const int items = nrows * pairs;
    // Warp-uniform trip count, so the row groups of a warp reduce together.
    for (int base = 0; base < items; base += blockDim.x) {
        if (base + (tid & ~31) >= items) continue;  // this warp has no pair in this pass
        const int i = base + tid;
        int r = 0, lo = INT_MAX, hi = -1;
        TileStat t[2] = {{256u, 0u, 0u}, {256u, 0u, 0u}};
        if (i < items) {
            r = i / pairs;
            const int pair = i - r * pairs;
            const int ty = ty0 + r;
            tile_pair_stats(gray, stride, W, H, ty, pair, vec16, &t[0], &t[1]);
#pragma unroll
            for (int k = 0; k < 2; ++k) {
                if (t[k].mn > 255u) continue;  // no second tile in this pair
                const int tx = 2 * pair + k;
                const int idx = ty * tw + tx;
                d.tile_min[idx] = static_cast<uint8_t>(t[k].mn);
                d.tile_max[idx] = static_cast<uint8_t>(t[k].mx);
                if (static_cast<int>(t[k].mx - t[k].mn) >= kMinTileContrast) {
                    lo = min(lo, tx);
                    hi = max(hi, tx);
                }
            }
        }
        // Histogram counts, one shared-memory atomic per distinct bin of the
        // warp: flat regions give most tiles of a row the same span and mean.
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const bool valid = i < items && t[k].mn <= 255u;
            const uint32_t span_bin = valid ? ((t[k].mx - t[k].mn) & 0xffu) : kNone;
            const uint32_t mean_bin = valid ? (t[k].mean >> 2) : kNone;
            const unsigned sp = __match_any_sync(kFull, span_bin);
            const unsigned mp = __match_any_sync(kFull, mean_bin);
            const int me = tid & 31;
            if (valid && me == __ffs(sp) - 1) atomicAdd(&s_span[span_bin], static_cast<uint32_t>(__popc(sp)));
            if (valid && me == __ffs(mp) - 1) atomicAdd(&s_mean[mean_bin], static_cast<uint32_t>(__popc(mp)));
        }
        const unsigned peers = __match_any_sync(kFull, r);
        lo = __reduce_min_sync(peers, lo);
        hi = __reduce_max_sync(peers, hi);
        if (hi >= 0 && (tid & 31) == __ffs(peers) - 1) {
            atomicMin(&s_lo[r], lo);
            atomicMax(&s_hi[r], hi);
        }
    }
    __syncthreads();
    if (tid < nrows) {
        const int ty = ty0 + tid;
        const int hi = s_hi[tid];
        d.row_lo[ty] = hi >= 0 ? s_lo[tid] : -1;
        d.row_hi[ty] = hi;
        if (hi >= 0) {
            atomicMax(&st->top_enc, static_cast<uint32_t>(d.tile_h - ty));
            atomicMax(&st->bottom_enc, static_cast<uint32_t>(ty + 1));
        }
    }
    if (s_span[tid]) atomicAdd(&st->span_hist[tid], s_span[tid]);
    if (tid < 64 && s_mean[tid]) atomicAdd(&st->mean_hist[tid], s_mean[tid]);
}

// ===========================================================================
// 2. Pooled threshold, binarization of the row band, run extraction and the
//    band-local connected components, for one band of 8 rows; warp w owns
//    row y0 + w.
//
//    The runs of a band are labelled in shared memory (same-row fragments and
//    8-connected runs of consecutive rows inside the band, by hooking and
//    flattening rounds), and area / bbox are aggregated per band-local root
//    with shared-memory atomics.  Global memory then receives one parent
//    link per run (to its band-local root) and one aggregate per band-local
//    root; k_merge only unions across band boundaries and k_region_stats
//    folds band roots into global roots.  The
//    local root is the band's smallest slot of the component, so every root
//    is still the component's smallest slot id (reference invariant,
//    gpu_detector.cu:398-421).  A band with more than `cap` runs (a launch
//    shape, 256..2048) is cut into row segments of at most `cap` runs,
//    labelled one after another, and k_merge also joins each segment's
//    first row to the row above; only a single row longer than `cap` sends
//    the band back to one root per run and full merging in k_merge.
// ===========================================================================

__device__ __forceinline__ void stage_binarize(const BatchDesc* __restrict__ b, const FrameIO* __restrict__ io, int fi,
                               int ty, int cap, int bits_words, BinSmem& sm, uint32_t* s_dyn) {
    uint32_t* sm_run = s_dyn;
    uint32_t* sm_par = s_dyn + cap;
    uint32_t* sm_area = s_dyn + 2 * cap;
    uint32_t* sm_minx = s_dyn + 3 * cap;
    uint32_t* sm_maxx = s_dyn + 4 * cap;
    uint32_t* sm_rows = s_dyn + 5 * cap;
    uint32_t* sm_bits = s_dyn + 6 * cap;  // kTile rows of bits_words words
    uint8_t* sm_row = reinterpret_cast<uint8_t*>(sm_bits + kTile * bits_words);  // cap: row of each run
    uint8_t* s_thresh = sm.thresh;
    uint8_t* s_vmin = sm.vmin;
    uint8_t* s_vmax = sm.vmax;
    uint32_t* s_rowtot = sm.rowtot;
    uint32_t* s_rowoff = sm.rowoff;

    const int tid = threadIdx.x;
    const FrameDesc& d = b->f[fi];
    FrameState* st = d.state;
    const int W = d.width, H = d.height, tw = d.tile_w, th = d.tile_h, words = d.words;
    const int y0 = ty * kTile;
    const int rows = min(kTile, H - y0);
    const uint32_t row_cap = static_cast<uint32_t>(d.row_cap);
    const uint32_t band_base = static_cast<uint32_t>(y0) * row_cap;

    const int top = th - static_cast<int>(st->top_enc);
    const int bottom = static_cast<int>(st->bottom_enc) - 1;
    const bool on = bottom >= 0 && ty >= top - 1 && ty <= bottom + 1;
    // Frame references from the complete histograms (reference
    // k_tile_reference :174-230): every band that thresholds computes them,
    // and band 0 also records them and the ROI row count (:2117).
    if (on || ty == 0) {
        frame_references(st->span_hist, st->mean_hist, sm.ref, &sm.refs[0], &sm.refs[1]);
        __syncthreads();
        if (ty == 0 && tid == 0) {
            st->ref[0] = sm.refs[0];
            st->ref[1] = sm.refs[1];
            st->counts[4] = roi_tile_rows(st->top_enc, st->bottom_enc, th);
        }
    }
    if (!on) {
        for (int i = tid; i < rows * words; i += blockDim.x) {
            d.bits[static_cast<int64_t>(y0 + i / words) * words + i % words] = 0xffffffffu;
        }
        if (tid < rows) d.row_count[y0 + tid] = 0;
        if (tid == 0) {
            d.lroot_count[ty] = 0;
            d.band_mode[ty] = 0;
        }
        return;
    }

    // Row band: contrasting tiles +- 4, or the whole row (reference :345-355).
    const int lo = d.row_lo[ty], hi = d.row_hi[ty];
    const int start = lo < 0 ? 0 : max(0, lo - 4);
    const int end = lo < 0 ? tw - 1 : min(tw - 1, hi + 4);
    const int wx_lo = start >> 2;
    const int wx_hi = end >> 2;

    // Pooled thresholds (reference k_tile_threshold :237-270).
    const uint32_t ref0 = sm.refs[0], ref1 = sm.refs[1];
    const int floor_contrast = max(kMinTileContrast, static_cast<int>((ref0 * 3) / 2));
    const int t_end = min(4 * wx_hi + 3, tw - 1);
    // The 3x3 window min/max, separably: columns over the three tile rows
    // (coalesced loads into shared memory), then three columns.
    const int c_lo = max(4 * wx_lo - 1, 0), c_hi = min(t_end + 1, tw - 1);
    for (int xx = c_lo + tid; xx <= c_hi; xx += blockDim.x) {
        int mn = 255, mx = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            const int yy = ty + dy;
            if (yy < 0 || yy >= th) continue;
            mn = min(mn, static_cast<int>(d.tile_min[yy * tw + xx]));
            mx = max(mx, static_cast<int>(d.tile_max[yy * tw + xx]));
        }
        s_vmin[xx] = static_cast<uint8_t>(mn);
        s_vmax[xx] = static_cast<uint8_t>(mx);
    }
    __syncthreads();
    for (int t = 4 * wx_lo + tid; t <= t_end; t += blockDim.x) {
        int mn = 255, mx = 0;
        for (int dx = -1; dx <= 1; ++dx) {
            const int xx = t + dx;
            if (xx < 0 || xx >= tw) continue;
            mn = min(mn, static_cast<int>(s_vmin[xx]));
            mx = max(mx, static_cast<int>(s_vmax[xx]));
        }
        int thr = static_cast<int>(ref1);
        if (mx - mn >= floor_contrast) thr = (mn + mx + 1) >> 1;
        s_thresh[t] = static_cast<uint8_t>(thr);
    }
    if (tid < kTile) s_rowtot[tid] = 0;
    __syncthreads();

    const int w = tid >> 5, lane = tid & 31;
    const uint8_t* gray = io[fi].gray;
    const int64_t stride = io[fi].stride;
    const bool vec = ((reinterpret_cast<uintptr_t>(gray) | static_cast<uintptr_t>(stride)) & 15u) == 0;
    const int per = (words + 31) >> 5;
    const int c0 = lane * per;
    const int c1 = min(c0 + per, words);
    uint32_t first_index = 0;  // exclusive prefix of this lane's fragments in its row
    if (w < rows) {
        const int y = y0 + w;
        const uint8_t* row = gray + static_cast<int64_t>(y) * stride;
        for (int wx = lane; wx < words; wx += 32) {
            uint32_t m = 0xffffffffu;
            if (wx >= wx_lo && wx <= wx_hi) {
                const int x = wx << 5;
                if (vec && x + 32 <= W) {
                    const uint4 a = *reinterpret_cast<const uint4*>(row + x);
                    const uint4 c = *reinterpret_cast<const uint4*>(row + x + 16);
                    const int t0 = x >> 3;
                    const uint32_t q0 = s_thresh[t0] * 0x01010101u, q1 = s_thresh[t0 + 1] * 0x01010101u;
                    const uint32_t q2 = s_thresh[t0 + 2] * 0x01010101u, q3 = s_thresh[t0 + 3] * 0x01010101u;
                    m = white_bits4(a.x, q0) | (white_bits4(a.y, q0) << 4) |
                        (white_bits4(a.z, q1) << 8) | (white_bits4(a.w, q1) << 12) |
                        (white_bits4(c.x, q2) << 16) | (white_bits4(c.y, q2) << 20) |
                        (white_bits4(c.z, q3) << 24) | (white_bits4(c.w, q3) << 28);
                } else {
                    m = 0u;
                    for (int k = 0; k < 32; ++k) {
                        const int xx = x + k;
                        const bool white = xx >= W || row[xx] > s_thresh[xx >> 3];
                        m |= (white ? 1u : 0u) << k;
                    }
                }
            }
            d.bits[static_cast<int64_t>(y) * words + wx] = m;
            sm_bits[w * bits_words + wx] = m;
        }
        __syncwarp();
        // Fragments per lane, then the row's prefix (reference :448-470).
        uint32_t cnt = 0;
        for (int c = c0; c < c1; ++c) {
            const uint32_t m = sm_bits[w * bits_words + c];
            cnt += __popc(~m & ((m << 1) | 1u));
        }
        uint32_t incl = cnt;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t n = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += n;
        }
        first_index = incl - cnt;
        const uint32_t total = __shfl_sync(kFull, incl, 31);
        if (lane == 0) {
            const uint32_t kept = min(total, row_cap);
            d.row_count[y] = kept;
            s_rowtot[w] = kept;
        }
    }
    __syncthreads();
    if (tid == 0) {
        uint32_t off = 0;
        for (int r = 0; r < kTile; ++r) {
            s_rowoff[r] = off;
            off += s_rowtot[r];
        }
        s_rowoff[kTile] = off;
        sm.nroots = 0;
        atomicAdd(&st->counts[2], off);
        // Row segments that fit `cap` runs: a segment starts at row r > 0
        // (bit r) where adding row r would exceed the cap.  A row longer
        // than the cap by itself sends the band to the fallback.
        uint32_t mask = 0, cum = 0;
        bool fits = true;
        for (int r = 0; r < kTile; ++r) {
            const uint32_t n = s_rowtot[r];
            if (n > static_cast<uint32_t>(cap)) fits = false;
            if (cum > 0 && cum + n > static_cast<uint32_t>(cap)) {
                mask |= 1u << r;
                cum = 0;
            }
            cum += n;
        }
        sm.segmask = fits ? mask : kNone;
    }
    __syncthreads();
    const uint32_t band_total = s_rowoff[kTile];
    const uint32_t segmask = sm.segmask;
    const bool fallback = segmask == kNone;
    const bool single = segmask == 0u;  // the whole band fits: runs go straight to shared memory

    // Emit the runs (reference :472-503).
    if (w < rows) {
        const int y = y0 + w;
        const uint32_t slot_base = static_cast<uint32_t>(y) * row_cap;
        uint32_t index = first_index;
        for (int c = c0; c < c1; ++c) {
            const uint32_t m = sm_bits[w * bits_words + c];
            uint32_t starts = ~m & ((m << 1) | 1u);
            const int last = min(31, W - 1 - (c << 5));
            while (starts) {
                const int s = __ffs(starts) - 1;
                starts &= starts - 1u;
                const int x0 = (c << 5) + s;
                if (x0 < W && index < row_cap) {
                    const int next_white = __ffs(m >> s);
                    int e = next_white ? (s + next_white - 2) : last;
                    e = min(e, last);
                    const int x1 = (c << 5) + e;
                    const uint32_t id = slot_base + index;
                    const uint32_t packed = (static_cast<uint32_t>(x0) & 0xffffu) | (static_cast<uint32_t>(x1) << 16);
                    d.runs[id] = packed;
                    if (single) {
                        const uint32_t li = s_rowoff[w] + index;
                        sm_run[li] = packed;
                        sm_par[li] = li;
                        sm_row[li] = static_cast<uint8_t>(w);
                    } else if (fallback) {
                        // Every run is its own band root.
                        d.parent[id] = id;
                        d.area[id] = static_cast<uint32_t>(x1 - x0 + 1);
                        reinterpret_cast<uint4*>(d.bbox)[id] = make_uint4(x0, y, x1, y);
                        d.lroots[band_base + s_rowoff[w] + index] = id;
                    }
                }
                ++index;
            }
        }
    }
    if (fallback) {
        if (tid == 0) {
            d.lroot_count[ty] = band_total;
            d.band_mode[ty] = 1;
        }
        return;
    }
    __syncthreads();

    // Band-local components, one row segment at a time (one segment when the
    // band fits).  Local index i of a segment = band index seg_off + i.
    for (int r0 = 0; r0 < kTile;) {
        int r1 = r0 + 1;
        while (r1 < kTile && !((segmask >> r1) & 1u)) ++r1;
        const uint32_t seg_off = s_rowoff[r0];
        const uint32_t seg_n = s_rowoff[r1] - seg_off;
        for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
            if (!single) {
                int row = 0;
                while (row + 1 < kTile && s_rowoff[row + 1] <= seg_off + i) ++row;
                sm_run[i] = d.runs[static_cast<int64_t>(y0 + row) * row_cap + (seg_off + i - s_rowoff[row])];
                sm_par[i] = i;
                sm_row[i] = static_cast<uint8_t>(row);
            }
            sm_minx[i] = 0xffffffffu;
            sm_maxx[i] = 0u;
            sm_rows[i] = 0u;
        }
        __syncthreads();

        // Unions inside the segment (the reference's k_merge_runs rules).
        // First the same-row rule: consecutive fragments that touch (a run
        // cut at word boundaries, or runs one pixel apart) form one group,
        // and every fragment points straight at the group's first fragment.
        // Linking each fragment to its left neighbour instead builds chains
        // as long as the row, which every later find walks.  Row 0 of the
        // frame is never merged, not even its word-split fragments
        // (reference k_merge_runs :514 returns for y <= 0).
        if (w >= r0 && w < r1 && w < rows && y0 + w > 0) {
            const uint32_t n = s_rowtot[w];
            const uint32_t base = s_rowoff[w] - seg_off;
            uint32_t carry = 0;  // group head of the previous chunk's last fragment
            for (uint32_t c = 0; c < n; c += 32) {
                const uint32_t i = c + static_cast<uint32_t>(lane);
                bool head = true;
                if (i < n && i > 0) {
                    const int x0 = static_cast<int>(sm_run[base + i] & 0xffffu);
                    const int px1 = static_cast<int>(sm_run[base + i - 1] >> 16);
                    head = px1 + 1 < x0;
                }
                const uint32_t upto = __ballot_sync(kFull, head) & (kFull >> (31 - lane));
                const uint32_t h = upto ? c + 31u - static_cast<uint32_t>(__clz(upto)) : carry;
                if (i < n) sm_par[base + i] = base + h;
                carry = __shfl_sync(kFull, h, 31);
            }
        }
        // Then the rows meet: run i of row r > r0 overlaps (8-connected) the
        // runs [first, first + count) of row r - 1, kept in sm_area[i] until
        // the roots pass needs it.
        for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
            const int row = sm_row[i];
            uint32_t list = 0;
            if (row > r0) {
                const uint32_t run = sm_run[i];
                const int x0 = static_cast<int>(run & 0xffffu);
                const int x1 = static_cast<int>(run >> 16);
                const uint32_t pbase = s_rowoff[row - 1] - seg_off;
                const int prev_n = static_cast<int>(s_rowtot[row - 1]);
                int lo2 = 0, hi2 = prev_n - 1, first = prev_n;
                while (lo2 <= hi2) {
                    const int mid = (lo2 + hi2) >> 1;
                    if (static_cast<int>(sm_run[pbase + mid] >> 16) >= x0 - 1) {
                        first = mid;
                        hi2 = mid - 1;
                    } else {
                        lo2 = mid + 1;
                    }
                }
                int k = first;
                while (k < prev_n && static_cast<int>(sm_run[pbase + k] & 0xffffu) <= x1 + 1) ++k;
                list = (pbase + static_cast<uint32_t>(first)) | (static_cast<uint32_t>(k - first) << 16);
            }
            sm_area[i] = list;
        }
        __syncthreads();

        // Components by hooking and flattening rounds.  A round hooks, for
        // every overlapping pair with different parents, the larger parent
        // under the smaller one (atomicMin), then flattens the forest, so
        // every round starts from roots.  Parents only decrease and always
        // stay in the component, so the rounds end; the last one finds every
        // pair under one root, which is the component's smallest index, as
        // with the reference's union-find.  Each round merges every tree with
        // a neighbour: 3-5 rounds on 8-row bands of camera frames, where
        // concurrent union-find walked chains of hundreds of links.
        for (;;) {
            int hooked = 0;
            for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
                const uint32_t list = sm_area[i];
                const uint32_t a = sm_par[i];
                for (uint32_t k = list & 0xffffu, k_end = k + (list >> 16); k < k_end; ++k) {
                    const uint32_t p = sm_par[k];
                    if (p != a) {
                        atomicMin(&sm_par[max(a, p)], min(a, p));
                        hooked = 1;
                    }
                }
            }
            if (!__syncthreads_or(hooked)) break;
            // Flatten in one pass: every entry walks to its root.  No hook
            // runs meanwhile, and a concurrent write only ever shortcuts a
            // walk to an ancestor.
            for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
                uint32_t r = sm_par[i];
                for (uint32_t q = sm_par[r]; q != r; q = sm_par[r]) r = q;
                sm_par[i] = r;
            }
            __syncthreads();
        }
        for (uint32_t i = tid; i < seg_n; i += blockDim.x) sm_area[i] = 0u;
        __syncthreads();

        // Segment roots (its smallest slot) and their area / bbox.
        for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
            const uint32_t r = sm_par[i];
            const int row = sm_row[i];
            const uint32_t run = sm_run[i];
            const uint32_t x0 = run & 0xffffu, x1 = run >> 16;
            atomicAdd(&sm_area[r], x1 - x0 + 1);
            atomicMin(&sm_minx[r], x0);
            atomicMax(&sm_maxx[r], x1);
            atomicOr(&sm_rows[r], 1u << row);
            // parent link = the local root's slot
            const int rrow = sm_row[r];
            const uint32_t slot = static_cast<uint32_t>(y0 + row) * row_cap + (seg_off + i - s_rowoff[row]);
            const uint32_t rslot = static_cast<uint32_t>(y0 + rrow) * row_cap + (seg_off + r - s_rowoff[rrow]);
            d.parent[slot] = rslot;
        }
        __syncthreads();
        for (uint32_t i = tid; i < seg_n; i += blockDim.x) {
            if (sm_par[i] != i) continue;
            const int row = sm_row[i];
            const uint32_t slot = static_cast<uint32_t>(y0 + row) * row_cap + (seg_off + i - s_rowoff[row]);
            const uint32_t rm = sm_rows[i];
            d.area[slot] = sm_area[i];
            reinterpret_cast<uint4*>(d.bbox)[slot] =
                make_uint4(sm_minx[i], static_cast<uint32_t>(y0 + __ffs(rm) - 1), sm_maxx[i],
                           static_cast<uint32_t>(y0 + 31 - __clz(rm)));
            d.lroots[band_base + atomicAdd(&sm.nroots, 1u)] = slot;
        }
        __syncthreads();
        r0 = r1;
    }
    if (tid == 0) {
        d.lroot_count[ty] = sm.nroots;
        d.band_mode[ty] = segmask;  // bit r: row r starts a segment (k_merge joins it to row r - 1)
    }
}

// ===========================================================================
// 3. Unions across band boundaries: the first row of a band against the last
//    row of the band above; every row of a fallback band (the reference's
//    k_merge_runs :509-557 rules).
// ===========================================================================
__device__ __forceinline__ void merge_run_with_row_above(uint32_t* parent, const uint32_t* cur,
                                                         const uint32_t* prev, int i, int prev_n,
                                                         uint32_t cur_base, uint32_t prev_base,
                                                         bool same_row) {
    const uint32_t run = cur[i];
    const int x0 = static_cast<int>(run & 0xffffu);
    const int x1 = static_cast<int>(run >> 16);
    if (same_row && i > 0) {
        const int px1 = static_cast<int>(cur[i - 1] >> 16);
        if (px1 + 1 >= x0) uf_union(parent, cur_base + i, cur_base + i - 1);
    }
    if (prev_n == 0) return;
    int lo = 0, hi = prev_n - 1, first = prev_n;
    while (lo <= hi) {
        const int mid = (lo + hi) >> 1;
        if (static_cast<int>(prev[mid] >> 16) >= x0 - 1) {
            first = mid;
            hi = mid - 1;
        } else {
            lo = mid + 1;
        }
    }
    for (int k = first; k < prev_n; ++k) {
        const int px0 = static_cast<int>(prev[k] & 0xffffu);
        if (px0 > x1 + 1) break;
        uf_union(parent, cur_base + i, prev_base + k);
    }
}

__device__ __forceinline__ void stage_merge(const BatchDesc* __restrict__ b, int fi, int ty, int row_cap_max,
                            uint32_t* s_dyn) {
    const FrameDesc& d = b->f[fi];
    const int row_cap = d.row_cap;
    uint32_t* parent = d.parent;
    const uint32_t mode = d.band_mode[ty];
    if (!(mode & 1u)) {
        // Band-local unions are done: the first row of the band, and the
        // first row of every further segment (bit r of the mode), meet the
        // row above.  Both rows are staged in shared memory (the searches
        // run there); their runs are spread over the whole CTA.
        uint32_t* s_prev = s_dyn;
        uint32_t* s_cur = s_dyn + row_cap_max;
        for (uint32_t starts = mode | 1u; starts; starts &= starts - 1u) {
            const int y = ty * kTile + __ffs(starts) - 1;
            if (y <= 0 || y >= d.height) continue;  // uniform over the CTA
            const int n = static_cast<int>(d.row_count[y]);
            const int prev_n = static_cast<int>(d.row_count[y - 1]);
            const uint32_t* cur = d.runs + static_cast<int64_t>(y) * row_cap;
            const uint32_t* prev = d.runs + static_cast<int64_t>(y - 1) * row_cap;
            for (int i = threadIdx.x; i < prev_n; i += blockDim.x) s_prev[i] = prev[i];
            for (int i = threadIdx.x; i < n; i += blockDim.x) s_cur[i] = cur[i];
            __syncthreads();
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                merge_run_with_row_above(parent, s_cur, s_prev, i, prev_n,
                                         static_cast<uint32_t>(y * row_cap),
                                         static_cast<uint32_t>((y - 1) * row_cap), false);
            }
            // The next pair reuses the buffers.  After the last pair, threads
            // without runs leave at once instead of waiting for the unions.
            if (starts & (starts - 1u)) __syncthreads();
        }
        return;
    }
    // Fallback band: every row, one warp per row.
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int y = ty * kTile + w;
    if (y <= 0 || y >= d.height) return;
    const int n = static_cast<int>(d.row_count[y]);
    const int prev_n = static_cast<int>(d.row_count[y - 1]);
    const uint32_t* cur = d.runs + static_cast<int64_t>(y) * row_cap;
    const uint32_t* prev = d.runs + static_cast<int64_t>(y - 1) * row_cap;
    for (int i = lane; i < n; i += 32) {
        merge_run_with_row_above(parent, cur, prev, i, prev_n, static_cast<uint32_t>(y * row_cap),
                                 static_cast<uint32_t>((y - 1) * row_cap), true);
    }
}

// ===========================================================================
// 4. Area and bounding box per global root: each band root adds its
//    aggregate to its global root (reference k_region_stats :562-586 sums the
//    same quantities run by run).
// ===========================================================================
__device__ __forceinline__ void stage_region(const BatchDesc* __restrict__ b, int fi, int ty) {
    const FrameDesc& d = b->f[fi];
    const uint32_t n = d.lroot_count[ty];
    const uint32_t* list = d.lroots + static_cast<int64_t>(ty) * kTile * d.row_cap;
    const uint32_t lane = threadIdx.x & 31u;
    // Warp-uniform sweep: lanes folding into the same global root combine
    // their sums and extremes first (order-free: integer adds, min, max), so
    // a component crossing many bands -- the background -- takes one set of
    // atomics per warp instead of one per band root.
    for (uint32_t base = threadIdx.x & ~31u; base < n; base += blockDim.x) {
        const uint32_t k = base + lane;
        uint32_t s = 0, g = 0;
        bool fold = false;
        if (k < n) {
            s = list[k];
            // All unions are done: walk to the root, halving the path for
            // the other bands' walks (the band root is relinked below).
            g = uf_root_halving(d.parent, s);
            fold = g != s;
        }
        const unsigned want = __ballot_sync(kFull, fold);
        if (!want) continue;
        uint32_t area = 0, x0 = 0xffffffffu, y0 = 0xffffffffu, x1 = 0, y1 = 0;
        if (fold) {
            d.parent[s] = g;  // later label walks take two hops
            const uint4 bb = reinterpret_cast<const uint4*>(d.bbox)[s];
            area = d.area[s];
            x0 = bb.x;
            y0 = bb.y;
            x1 = bb.z;
            y1 = bb.w;
        }
        const unsigned peers = __match_any_sync(kFull, fold ? g : 0xffffffffu);
        if (!fold) continue;
        area = __reduce_add_sync(peers, area);
        x0 = __reduce_min_sync(peers, x0);
        y0 = __reduce_min_sync(peers, y0);
        x1 = __reduce_max_sync(peers, x1);
        y1 = __reduce_max_sync(peers, y1);
        if (lane == static_cast<uint32_t>(__ffs(peers) - 1)) {
            atomicAdd(&d.area[g], area);
            atomicMin(&d.bbox[g * 4 + 0], x0);
            atomicMin(&d.bbox[g * 4 + 1], y0);
            atomicMax(&d.bbox[g * 4 + 2], x1);
            atomicMax(&d.bbox[g * 4 + 3], y1);
        }
    }
}

// ===========================================================================
// 5. Root labels, the tag-like filter and ordered ranks.  A candidate's
//    flattened position is (area bin, band, row, slot) order, which is
//    ascending root id inside a bin; the reference orders a bin by atomicAdd
//    arrival (k_collect_candidates :591-638).
// ===========================================================================
__device__ __forceinline__ int candidate_bin(const FrameDesc& d, uint32_t idx, int split_px,
                                             bool* big) {
    const int a = static_cast<int>(d.area[idx]);
    const uint4 bb = reinterpret_cast<const uint4*>(d.bbox)[idx];
    *big = big_candidate(bb, split_px);
    if (a < d.min_cluster_pixels) return -1;
    const int x0 = static_cast<int>(bb.x), y0 = static_cast<int>(bb.y);
    const int x1 = static_cast<int>(bb.z), y1 = static_cast<int>(bb.w);
    const int bw = x1 - x0 + 1;
    const int bh = y1 - y0 + 1;
    if (bw < d.min_tag_pixels || bh < d.min_tag_pixels) return -1;
    if (x0 <= 0 || y0 <= 0 || x1 >= d.width - 1 || y1 >= d.height - 1) return -1;
    if (bw > 6 * bh || bh > 6 * bw) return -1;
    const float fill = static_cast<float>(a) / static_cast<float>(bw * bh);
    if (fill < 0.18f || fill > 0.95f) return -1;
    const int log2_area = 31 - __clz(static_cast<uint32_t>(a));
    return 63 - min(log2_area, 63);
}

__device__ __forceinline__ uint32_t band_slot(const uint32_t* rowoff, int y0, uint32_t row_cap,
                                              uint32_t i) {
    int row = 0;
    while (row + 1 < kTile && rowoff[row + 1] <= i) ++row;
    return static_cast<uint32_t>(y0 + row) * row_cap + (i - rowoff[row]);
}

// One CTA per band, 256 runs at a time in slot order: root labels, the
// tag-like filter, and each candidate's rank among the band's candidates
// of its area bin.
__device__ __forceinline__ bool stage_cand(const BatchDesc* __restrict__ b, int fi, int ty, int split_px, CandSmem& sm,
                           uint32_t* s_cprefix) {
    uint32_t* s_rowoff = sm.rowoff;
    uint32_t (*s_wbin)[64] = sm.wbin;
    uint32_t* s_run = sm.run;
    uint32_t (*s_chunk)[64] = sm.chunk;
    uint32_t* s_total = sm.total;
    uint32_t* s_base = sm.base;
    uint32_t* s_warp_sum = sm.warp_sum;
    const int tid = threadIdx.x;
    const FrameDesc& d = b->f[fi];
    FrameState* st = d.state;
    const int y0 = ty * kTile;
    const uint32_t row_cap = static_cast<uint32_t>(d.row_cap);
    if (tid == 0) {
        uint32_t off = 0;
        for (int r = 0; r < kTile; ++r) {
            s_rowoff[r] = off;
            off += y0 + r < d.height ? d.row_count[y0 + r] : 0u;
        }
        s_rowoff[kTile] = off;
    }
    if (tid < 64) s_run[tid] = 0;
    if (tid == 0) sm.ncand = 0;
    __syncthreads();
    const uint32_t total = s_rowoff[kTile];
    const int w = tid >> 5, lane = tid & 31;
    // The band's candidate roots are listed in its lroots range (free since
    // k_region_stats), and their bin / rank words at the same positions of
    // cand_meta, for the frame's last CTA to place.
    uint32_t* band_list = d.lroots + static_cast<int64_t>(ty) * kTile * row_cap;
    uint32_t* band_meta = d.cand_meta + static_cast<int64_t>(ty) * kTile * row_cap;
    // Up to four chunks of 256 runs at a time: their label and root loads are
    // issued together, then the chunks are ranked one after another in slot
    // order, as before.
    constexpr int kChunks = 4;
    for (uint32_t gbase = 0; gbase < total; gbase += kChunks * blockDim.x) {
        int bins[kChunks];
        bool bigs[kChunks];
        uint32_t slots[kChunks], hop[kChunks];
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            const uint32_t i = gbase + u * blockDim.x + tid;
            bins[u] = -1;
            bigs[u] = false;
            slots[u] = 0;
            hop[u] = 0;
            if (i < total) {
                slots[u] = band_slot(s_rowoff, y0, row_cap, i);
                hop[u] = __ldcg(d.parent + slots[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            if (gbase + u * blockDim.x + tid < total) {
                // Two hops reach the root: a run's parent is a band root (or
                // a root above it after k_merge's path halving), and
                // k_region_stats pointed every band root at its component's
                // root.
                hop[u] = __ldcg(d.parent + hop[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            if (gbase + u * blockDim.x + tid < total) {
                d.parent[slots[u]] = hop[u];
                if (hop[u] == slots[u]) bins[u] = candidate_bin(d, slots[u], split_px, &bigs[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
            if (gbase + u * blockDim.x >= total) break;  // uniform over the CTA
            const int bin = bins[u];
            const bool big = bigs[u];
            const uint32_t slot = slots[u];
            const uint32_t key = bin >= 0 ? static_cast<uint32_t>(bin) : 64u + lane;
            const uint32_t peers = __match_any_sync(kFull, key);
            const uint32_t rank = __popc(peers & lanemask_lt());
            s_wbin[w][lane] = 0;
            s_wbin[w][lane + 32] = 0;
            __syncthreads();
            if (bin >= 0 && rank == 0) s_wbin[w][bin] = __popc(peers);
            __syncthreads();
            uint32_t meta = kNone;
            if (bin >= 0) {
                uint32_t pos = s_run[bin] + rank;
                for (int w2 = 0; w2 < w; ++w2) pos += s_wbin[w2][bin];
                meta = (static_cast<uint32_t>(bin) << 24) | (big ? 1u << 23 : 0u) | pos;
            }
            __syncthreads();
            if (tid < 64) {
                uint32_t add = 0;
                for (int w2 = 0; w2 < 8; ++w2) add += s_wbin[w2][tid];
                s_run[tid] += add;
            }
            if (bin >= 0) {
                const uint32_t at = atomicAdd(&sm.ncand, 1u);
                band_list[at] = slot;
                band_meta[at] = meta;
            }
            __syncthreads();  // s_wbin is cleared for the next chunk
        }
    }
    __syncthreads();
    if (tid < 64) d.band_bins[ty * 64 + tid] = s_run[tid];
    if (tid == 0) d.lroot_count[ty] = sm.ncand;
    __threadfence();
    __syncthreads();
    if (tid == 0) sm.last = atomicAdd(&st->done_cands, 1u) == static_cast<uint32_t>(d.tile_h - 1);
    __syncthreads();
    if (!sm.last) return false;
    __threadfence();

    // Last band: exclusive prefix of every bin over the bands (in place).
    // Thread (segment q, bin) sums a quarter of the bands (loads coalesced
    // over the bins), the four segment sums are scanned per bin, and each
    // thread rewrites its quarter from its segment's offset.
    const int th = d.tile_h;
    const int bin = tid & 63;
    const int q = tid >> 6;
    const int per = (th + 3) >> 2;
    const int qb0 = min(th, q * per), qb1 = min(th, qb0 + per);
    // Both passes load eight bands at a time, so a quarter of a frame's
    // bands costs a few L2 round trips instead of one per band.
    constexpr int kBatch = 8;
    uint32_t sum = 0;
    for (int band = qb0; band < qb1; band += kBatch) {
        uint32_t v[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) v[k] = band + k < qb1 ? __ldcg(&d.band_bins[(band + k) * 64 + bin]) : 0u;
#pragma unroll
        for (int k = 0; k < kBatch; ++k) sum += v[k];
    }
    s_chunk[q][bin] = sum;
    __syncthreads();
    uint32_t carry = 0;
    for (int q2 = 0; q2 < q; ++q2) carry += s_chunk[q2][bin];
    if (q == 3) s_total[bin] = carry + sum;
    for (int band = qb0; band < qb1; band += kBatch) {
        uint32_t v[kBatch];
#pragma unroll
        for (int k = 0; k < kBatch; ++k) v[k] = band + k < qb1 ? __ldcg(&d.band_bins[(band + k) * 64 + bin]) : 0u;
#pragma unroll
        for (int k = 0; k < kBatch; ++k) {
            if (band + k < qb1) {
                d.band_bins[(band + k) * 64 + bin] = carry;
                carry += v[k];
            }
        }
    }
    __syncthreads();
    if (tid < 32) {
        // Exclusive scan of the 64 bin totals: lane l holds bins 2l, 2l + 1.
        const uint32_t t0 = s_total[2 * lane], t1 = s_total[2 * lane + 1];
        uint32_t incl = t0 + t1;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t n = __shfl_up_sync(kFull, incl, off);
            if (lane >= off) incl += n;
        }
        const uint32_t before = incl - t0 - t1;
        s_base[2 * lane] = before;
        s_base[2 * lane + 1] = before + t0;
        st->bin_base[2 * lane] = before;
        st->bin_base[2 * lane + 1] = before + t0;
        if (lane == 31) {
            st->counts[0] = incl;
            sm.limit = min(incl, static_cast<uint32_t>(d.max_candidates));
            st->n_candidates = sm.limit;
            sm.nbig = 0;
            sm.nsmall = 0;
        }
    }

    // Placement (reference k_order_candidates :642-654): candidate j of the
    // frame, flattened over the bands' lists, goes to bin base + earlier
    // bands' count in its bin + its rank in the band.  Block scan of the
    // per-band list lengths first.
    const int chunk = (th + blockDim.x - 1) / blockDim.x;
    const int cb0 = min(th, tid * chunk), cb1 = min(th, cb0 + chunk);
    uint32_t own = 0;
    for (int band = cb0; band < cb1; ++band) own += __ldcg(&d.lroot_count[band]);
    uint32_t incl = own;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t v = __shfl_up_sync(kFull, incl, off);
        if (lane >= off) incl += v;
    }
    if (lane == 31) s_warp_sum[w] = incl;
    __syncthreads();
    uint32_t before = incl - own;
    for (int w2 = 0; w2 < w; ++w2) before += s_warp_sum[w2];
    for (int band = cb0; band < cb1; ++band) {
        s_cprefix[band] = before;
        before += __ldcg(&d.lroot_count[band]);
    }
    if (tid == blockDim.x - 1) s_cprefix[th] = before;
    __syncthreads();
    const uint32_t all = s_cprefix[th];
    const uint32_t limit = sm.limit;
    // Four candidates per thread and pass, their loads in flight together:
    // slot and bin word (one position of both band lists), then the band's
    // bin prefix.
    constexpr int kUnroll = 4;
    for (uint32_t j0 = tid; j0 < all; j0 += kUnroll * blockDim.x) {
        uint32_t slot[kUnroll], meta[kUnroll], prev[kUnroll];
        int band[kUnroll];
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            const uint32_t j = j0 + u * blockDim.x;
            band[u] = -1;
            if (j < all) {
                int lo = 0, hi = th - 1;  // last band with s_cprefix[band] <= j
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_cprefix[mid] <= j) lo = mid; else hi = mid - 1;
                }
                band[u] = lo;
                const int64_t at = static_cast<int64_t>(lo) * kTile * row_cap + (j - s_cprefix[lo]);
                slot[u] = __ldcg(&d.lroots[at]);
                meta[u] = __ldcg(&d.cand_meta[at]);
            }
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            if (band[u] >= 0) prev[u] = __ldcg(&d.band_bins[band[u] * 64 + (meta[u] >> 24)]);
        }
#pragma unroll
        for (int u = 0; u < kUnroll; ++u) {
            if (band[u] < 0) continue;
            const uint32_t pos = s_base[meta[u] >> 24] + prev[u] + (meta[u] & 0x7fffffu);
            if (pos < limit) {
                d.candidates[pos] = slot[u];
                // The fit/decode work lists, split by size once here: big
                // candidates (a CTA each) from the front, the others (a warp
                // per family) from the back.
                if (meta[u] & (1u << 23)) {
                    d.fit_list[atomicAdd(&sm.nbig, 1u)] = pos;
                } else {
                    d.fit_list[d.max_candidates - 1 - static_cast<int>(atomicAdd(&sm.nsmall, 1u))] = pos;
                }
            }
        }
    }
    __syncthreads();
    if (tid == 0) {
        st->n_big = sm.nbig;
        st->n_small = sm.nsmall;
    }
    return true;
}

}  // namespace
}  // namespace bdgb
