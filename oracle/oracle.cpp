// CPU ORACLE -- test infrastructure, not part of the product.  See oracle.h
// for what it restates, how it is pinned and its two conventions.
//
// Built with -O2 -ffp-contract=off (oracle/Makefile).  Each function cites the
// reference lines (detector/src/gpu_detector.cu unless noted) it restates.

#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <vector>

#include "../bd-cudatag_gb300/csrc/detmath.h"

namespace {

#include "../bd-cudatag_gb300/csrc/families_data.inc"

const uint64_t kCodewords36h11[BD_CODEWORDS_36H11_COUNT] = {BD_CODEWORDS_36H11};
const uint64_t kCodewords16h5[BD_CODEWORDS_16H5_COUNT] = {BD_CODEWORDS_16H5};

struct Family {
    const char* name;
    int bits_per_side;
    int border_cells;
    int code_count;
    const uint64_t* codes;
};

const Family kFamilies[2] = {
    {"tag36h11", 6, 1, 587, kCodewords36h11},
    {"tag16h5", 4, 1, 30, kCodewords16h5},
};

constexpr int kTile = 8;
constexpr int kMinTileContrast = 12;
constexpr int kFitDirections = 32;
constexpr int kMaxBoundaryRows = 1024;
constexpr int kMaxHullVertices = 64;
constexpr int kFitIterations = 2;
constexpr int kFitProbeHalf = 24;
constexpr uint32_t kNone = 0xffffffffu;

inline int popc32(uint32_t v) { return __builtin_popcount(v); }
inline int popc64(uint64_t v) { return __builtin_popcountll(v); }
inline int ffs32(uint32_t v) { return v ? __builtin_ctz(v) + 1 : 0; }

struct Params {
    int family = 0;
    int width = 0, height = 0, stride = 0;
    int tile_w = 0, tile_h = 0, words = 0, row_cap = 0;
    int min_cluster_pixels = 0, min_tag_pixels = 0;
    int max_candidates = 0, max_detections = 0;
    int dim = 0, max_hamming = 0, code_count = 0;
    const uint64_t* codes = nullptr;
    int refine_edges = 0;
    float min_margin = 0.0f, sharpening = 0.0f;
};

int next_power_of_two(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

// Caps and geometry: gpu_detector.cu:1905-1943, detector.cpp:39-57, :97-110.
Params resolve(int family, int width, int height, int stride, const bd_config* config) {
    bd_config c;
    std::memset(&c, 0, sizeof(c));
    c.struct_size = sizeof(bd_config);
    c.max_hamming = -1;
    c.min_cluster_pixels = 24;
    c.min_tag_pixels = 8;
    c.max_detections = 64;
    c.max_candidates = 0;
    c.refine_edges = 1;
    c.use_cuda_graph = 1;
    c.min_decision_margin = 3.0f;
    c.decode_sharpening = 0.25f;
    if (config) c = *config;

    Params p;
    const Family& fam = kFamilies[family];
    p.family = family;
    p.width = width;
    p.height = height;
    p.stride = stride;
    p.tile_w = (width + kTile - 1) / kTile;
    p.tile_h = (height + kTile - 1) / kTile;
    p.words = (width + 31) / 32;
    p.row_cap = width / 2 + 2;
    p.min_cluster_pixels = std::max(c.min_cluster_pixels, 1);
    p.min_tag_pixels = std::max(c.min_tag_pixels, 4);
    p.max_detections = std::min(std::max(c.max_detections, 1), 256);
    p.max_hamming = c.max_hamming >= 0 ? std::min(c.max_hamming, 3) : (family == 0 ? 2 : 1);
    p.max_candidates =
        c.max_candidates > 0
            ? std::min(std::max(c.max_candidates, 16), 1024)
            : std::min(std::max(next_power_of_two((width * height) / 4096) * 3 / 2, 96), 1024);
    p.dim = fam.bits_per_side + 2 * fam.border_cells;
    p.code_count = fam.code_count;
    p.codes = fam.codes;
    p.refine_edges = c.refine_edges ? 1 : 0;
    p.min_margin = c.min_decision_margin;
    p.sharpening = c.decode_sharpening;
    return p;
}

struct DecodeOut {
    int32_t id;
    int32_t hamming;
    float margin;
    float corners[8];
};

}  // namespace

struct bdo_frame {
    Params p;
    std::vector<uint8_t> tile_min, tile_max, tile_mean, thresh, active;
    uint32_t span_hist[256];
    uint32_t mean_hist[64];
    uint32_t ref[2];
    std::vector<uint8_t> row_active;
    std::vector<int32_t> row_start, row_end;
    std::vector<uint32_t> bits, row_count, runs, parent, label, area, bbox;
    uint32_t counts[5];
    std::vector<uint32_t> candidates;
    std::vector<float> hull_quads, quads;
    std::vector<DecodeOut> decodes;
    std::vector<bd_detection> detections;
};

namespace {

// --- 1. tile threshold ------------------------------------------------------

// k_tile_stats :104-135
void tile_stats(const uint8_t* gray, bdo_frame& f) {
    const Params& p = f.p;
    const int T = p.tile_w * p.tile_h;
    f.tile_min.assign(T, 0);
    f.tile_max.assign(T, 0);
    f.tile_mean.assign(T, 0);
    for (int idx = 0; idx < T; ++idx) {
        const int tx = idx % p.tile_w, ty = idx / p.tile_w;
        const int x0 = tx * kTile, y0 = ty * kTile;
        const int x1 = std::min(x0 + kTile, p.width), y1 = std::min(y0 + kTile, p.height);
        int mn = 255, mx = 0, sum = 0, count = 0;
        for (int y = y0; y < y1; ++y) {
            const uint8_t* row = gray + static_cast<size_t>(y) * p.stride;
            for (int x = x0; x < x1; ++x) {
                const int v = row[x];
                mn = std::min(mn, v);
                mx = std::max(mx, v);
                sum += v;
                ++count;
            }
        }
        f.tile_min[idx] = static_cast<uint8_t>(mn);
        f.tile_max[idx] = static_cast<uint8_t>(mx);
        f.tile_mean[idx] = static_cast<uint8_t>(count > 0 ? (sum + count / 2) / count : 0);
    }
}

// k_tile_histograms :140-166 and k_tile_reference :174-230
void tile_reference(bdo_frame& f) {
    const int T = f.p.tile_w * f.p.tile_h;
    std::memset(f.span_hist, 0, sizeof(f.span_hist));
    std::memset(f.mean_hist, 0, sizeof(f.mean_hist));
    for (int i = 0; i < T; ++i) {
        const int span = static_cast<int>(f.tile_max[i]) - static_cast<int>(f.tile_min[i]);
        f.span_hist[span & 0xff] += 1;
        f.mean_hist[f.tile_mean[i] >> 2] += 1;
    }

    uint32_t span_total = 0;
    for (int i = 0; i < 256; ++i) span_total += f.span_hist[i];
    uint32_t span = 0;
    if (span_total > 0) {
        const uint32_t target = span_total / 4;
        uint32_t seen = 0;
        for (int i = 0; i < 256; ++i) {
            seen += f.span_hist[i];
            if (seen > target) {
                span = static_cast<uint32_t>(i);
                break;
            }
        }
    }
    f.ref[0] = span;

    const uint32_t* means = f.mean_hist;
    float total = 0.0f;
    float sum = 0.0f;
    for (int i = 0; i < 64; ++i) {
        total += static_cast<float>(means[i]);
        sum += static_cast<float>(i) * static_cast<float>(means[i]);
    }
    int otsu = 0;
    if (total > 0.0f) {
        float weight_below = 0.0f;
        float sum_below = 0.0f;
        float best = -1.0f;
        for (int i = 0; i < 64; ++i) {
            weight_below += static_cast<float>(means[i]);
            if (weight_below <= 0.0f) continue;
            const float weight_above = total - weight_below;
            if (weight_above <= 0.0f) break;
            sum_below += static_cast<float>(i) * static_cast<float>(means[i]);
            const float mean_below = sum_below / weight_below;
            const float mean_above = (sum - sum_below) / weight_above;
            const float delta = mean_below - mean_above;
            const float between = weight_below * weight_above * delta * delta;
            if (between > best) {
                best = between;
                otsu = i;
            }
        }
    }
    f.ref[1] = static_cast<uint32_t>(otsu * 4 + 2);
}

// k_tile_threshold :237-276
void tile_threshold(bdo_frame& f) {
    const Params& p = f.p;
    const int T = p.tile_w * p.tile_h;
    f.thresh.assign(T, 0);
    f.active.assign(T, 0);
    const int floor_contrast = std::max(kMinTileContrast, static_cast<int>((f.ref[0] * 3) / 2));
    for (int idx = 0; idx < T; ++idx) {
        const int tx = idx % p.tile_w, ty = idx / p.tile_w;
        int mn = 255, mx = 0;
        for (int dy = -1; dy <= 1; ++dy) {
            const int y = ty + dy;
            if (y < 0 || y >= p.tile_h) continue;
            for (int dx = -1; dx <= 1; ++dx) {
                const int x = tx + dx;
                if (x < 0 || x >= p.tile_w) continue;
                mn = std::min(mn, static_cast<int>(f.tile_min[y * p.tile_w + x]));
                mx = std::max(mx, static_cast<int>(f.tile_max[y * p.tile_w + x]));
            }
        }
        int t = static_cast<int>(f.ref[1]);
        if (mx - mn >= floor_contrast) t = (mn + mx + 1) >> 1;
        f.thresh[idx] = static_cast<uint8_t>(t);
        const int own = static_cast<int>(f.tile_max[idx]) - static_cast<int>(f.tile_min[idx]);
        f.active[idx] = own >= kMinTileContrast ? 1u : 0u;
    }
}

// k_build_row_roi :282-357
void row_roi(bdo_frame& f) {
    const Params& p = f.p;
    f.row_active.assign(p.tile_h, 0);
    f.row_start.assign(p.tile_h, 0);
    f.row_end.assign(p.tile_h, -1);
    int top = p.tile_h, bottom = -1;
    for (int i = 0; i < p.tile_w * p.tile_h; ++i) {
        if (f.active[i]) {
            top = std::min(top, i / p.tile_w);
            bottom = std::max(bottom, i / p.tile_w);
        }
    }
    for (int ty = 0; ty < p.tile_h; ++ty) {
        if (bottom < 0 || ty < top - 1 || ty > bottom + 1) continue;
        int mn = p.tile_w, mx = -1;
        for (int x = 0; x < p.tile_w; ++x) {
            if (f.active[ty * p.tile_w + x]) {
                mn = std::min(mn, x);
                mx = std::max(mx, x);
            }
        }
        f.row_active[ty] = 1;
        f.counts[4] += 1;
        if (mx < 0) {
            f.row_start[ty] = 0;
            f.row_end[ty] = p.tile_w - 1;
        } else {
            f.row_start[ty] = std::max(0, mn - 4);
            f.row_end[ty] = std::min(p.tile_w - 1, mx + 4);
        }
    }
}

// --- 2. binarize :362-391 ---------------------------------------------------
void binarize(const uint8_t* gray, bdo_frame& f) {
    const Params& p = f.p;
    f.bits.assign(static_cast<size_t>(p.height) * p.words, 0);
    for (int y = 0; y < p.height; ++y) {
        const int ty = y >> 3;
        for (int wx = 0; wx < p.words; ++wx) {
            const int tile0 = wx << 2;
            const bool overlap = f.row_active[ty] != 0 && tile0 <= f.row_end[ty] &&
                                 tile0 + 3 >= f.row_start[ty];
            uint32_t mask = 0xffffffffu;
            if (overlap) {
                mask = 0;
                for (int lane = 0; lane < 32; ++lane) {
                    const int x = (wx << 5) + lane;
                    bool white = true;
                    if (x < p.width) {
                        const int t = f.thresh[ty * p.tile_w + (x >> 3)];
                        white = gray[static_cast<size_t>(y) * p.stride + x] > t;
                    }
                    if (white) mask |= 1u << lane;
                }
            }
            f.bits[static_cast<size_t>(y) * p.words + wx] = mask;
        }
    }
}

// --- 3-5. runs, union-find, component stats ---------------------------------

// Union-find with the reference's rule: the root of a component is its
// smallest slot id (uf_find / uf_union :398-421).  Sequential here, so the
// hooking order does not matter; only the partition and the min-id root do.
uint32_t find_root(std::vector<uint32_t>& parent, uint32_t x) {
    while (parent[x] != x) {
        parent[x] = parent[parent[x]];
        x = parent[x];
    }
    return x;
}

void unite(std::vector<uint32_t>& parent, uint32_t a, uint32_t b) {
    a = find_root(parent, a);
    b = find_root(parent, b);
    if (a == b) return;
    if (a < b)
        parent[b] = a;
    else
        parent[a] = b;
}

// k_find_runs :427-504
void find_runs(bdo_frame& f) {
    const Params& p = f.p;
    const size_t slots = static_cast<size_t>(p.height) * p.row_cap;
    f.row_count.assign(p.height, 0);
    f.runs.assign(slots, 0);
    f.parent.assign(slots, kNone);
    for (int y = 0; y < p.height; ++y) {
        if (!f.row_active[y >> 3]) continue;
        const uint32_t* row_bits = f.bits.data() + static_cast<size_t>(y) * p.words;
        uint32_t off = 0;
        std::vector<uint32_t> chunk_offsets(p.words);
        for (int c = 0; c < p.words; ++c) {
            const uint32_t mask = row_bits[c];
            const uint32_t starts = ~mask & ((mask << 1) | 1u);
            chunk_offsets[c] = off;
            off += static_cast<uint32_t>(popc32(starts));
        }
        const uint32_t total = std::min(off, static_cast<uint32_t>(p.row_cap));
        f.row_count[y] = total;
        f.counts[2] += total;
        for (int c = 0; c < p.words; ++c) {
            const uint32_t mask = row_bits[c];
            const uint32_t starts = ~mask & ((mask << 1) | 1u);
            for (int s = 0; s < 32; ++s) {
                if ((starts & (1u << s)) == 0u) continue;
                const int rank = popc32(starts & ((1u << s) - 1u));
                const int x0 = (c << 5) + s;
                if (x0 >= p.width) continue;
                const int last = std::min(31, p.width - 1 - (c << 5));
                const int next_white = ffs32(mask >> s);
                int e = next_white ? (s + next_white - 2) : last;
                e = std::min(e, last);
                const int x1 = (c << 5) + e;
                const int index = static_cast<int>(chunk_offsets[c]) + rank;
                if (index >= p.row_cap) continue;
                const uint32_t id = static_cast<uint32_t>(y * p.row_cap + index);
                f.runs[id] = (static_cast<uint32_t>(x0) & 0xffffu) |
                             ((static_cast<uint32_t>(x1) & 0xffffu) << 16);
                f.parent[id] = id;
            }
        }
    }
}

// k_merge_runs :509-557
void merge_runs(bdo_frame& f) {
    const Params& p = f.p;
    for (int y = 1; y < p.height; ++y) {
        if (!f.row_active[y >> 3]) continue;
        const int n = static_cast<int>(f.row_count[y]);
        const int prev_n = static_cast<int>(f.row_count[y - 1]);
        const uint32_t* cur = f.runs.data() + static_cast<size_t>(y) * p.row_cap;
        const uint32_t* prev = f.runs.data() + static_cast<size_t>(y - 1) * p.row_cap;
        const uint32_t cur_base = static_cast<uint32_t>(y * p.row_cap);
        const uint32_t prev_base = static_cast<uint32_t>((y - 1) * p.row_cap);
        for (int i = 0; i < n; ++i) {
            const int x0 = static_cast<int>(cur[i] & 0xffffu);
            const int x1 = static_cast<int>(cur[i] >> 16);
            if (i > 0) {
                const int px1 = static_cast<int>(cur[i - 1] >> 16);
                if (px1 + 1 >= x0) unite(f.parent, cur_base + i, cur_base + i - 1);
            }
            if (prev_n == 0) continue;
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
                unite(f.parent, cur_base + i, prev_base + k);
            }
        }
    }
}

// k_region_stats :562-586 (plus the flattened root label of every run)
void region_stats(bdo_frame& f) {
    const Params& p = f.p;
    const size_t slots = static_cast<size_t>(p.height) * p.row_cap;
    f.label.assign(slots, kNone);
    f.area.assign(slots, 0);
    f.bbox.assign(slots * 4, 0);
    for (size_t i = 0; i < slots; ++i) {
        f.bbox[i * 4 + 0] = kNone;
        f.bbox[i * 4 + 1] = kNone;
    }
    for (int y = 0; y < p.height; ++y) {
        if (!f.row_active[y >> 3]) continue;
        const int n = static_cast<int>(f.row_count[y]);
        for (int i = 0; i < n; ++i) {
            const uint32_t idx = static_cast<uint32_t>(y * p.row_cap + i);
            const uint32_t root = find_root(f.parent, idx);
            f.label[idx] = root;
            const uint32_t run = f.runs[idx];
            const uint32_t x0 = run & 0xffffu, x1 = run >> 16;
            f.area[root] += x1 - x0 + 1;
            f.bbox[root * 4 + 0] = std::min(f.bbox[root * 4 + 0], x0);
            f.bbox[root * 4 + 1] = std::min(f.bbox[root * 4 + 1], static_cast<uint32_t>(y));
            f.bbox[root * 4 + 2] = std::max(f.bbox[root * 4 + 2], x1);
            f.bbox[root * 4 + 3] = std::max(f.bbox[root * 4 + 3], static_cast<uint32_t>(y));
        }
    }
}

// --- 6. candidates: k_collect_candidates :591-638, k_order_candidates :642-654
// Canonical order: bins from the largest area down, root slot id ascending
// inside a bin (the reference's in-bin order comes from atomicAdd).
void collect_candidates(bdo_frame& f) {
    const Params& p = f.p;
    std::vector<std::vector<uint32_t>> bins(64);
    for (int y = 0; y < p.height; ++y) {
        if (!f.row_active[y >> 3]) continue;
        const int n = static_cast<int>(f.row_count[y]);
        for (int i = 0; i < n; ++i) {
            const uint32_t idx = static_cast<uint32_t>(y * p.row_cap + i);
            if (f.label[idx] != idx) continue;
            const int a = static_cast<int>(f.area[idx]);
            if (a < p.min_cluster_pixels) continue;
            const int x0 = static_cast<int>(f.bbox[idx * 4 + 0]);
            const int y0 = static_cast<int>(f.bbox[idx * 4 + 1]);
            const int x1 = static_cast<int>(f.bbox[idx * 4 + 2]);
            const int y1 = static_cast<int>(f.bbox[idx * 4 + 3]);
            const int bw = x1 - x0 + 1;
            const int bh = y1 - y0 + 1;
            if (bw < p.min_tag_pixels || bh < p.min_tag_pixels) continue;
            if (x0 <= 0 || y0 <= 0 || x1 >= p.width - 1 || y1 >= p.height - 1) continue;
            if (bw > 6 * bh || bh > 6 * bw) continue;
            const float fill = static_cast<float>(a) / static_cast<float>(bw * bh);
            if (fill < 0.18f || fill > 0.95f) continue;
            const int log2_area = 31 - __builtin_clz(static_cast<uint32_t>(a));
            const int bin = 63 - std::min(log2_area, 63);
            f.counts[0] += 1;
            bins[bin].push_back(idx);  // rows, then slots: ascending root id
        }
    }
    const uint32_t limit = std::min(f.counts[0], static_cast<uint32_t>(p.max_candidates));
    f.candidates.clear();
    for (int bin = 0; bin < 64 && f.candidates.size() < limit; ++bin) {
        for (uint32_t root : bins[bin]) {
            if (f.candidates.size() >= limit) break;
            f.candidates.push_back(root);
        }
    }
}

// --- 7. quad fit :659-1241 ----------------------------------------------------

inline uint32_t pack_point(int x, int y) {
    return (static_cast<uint32_t>(x) & 0xffffu) | (static_cast<uint32_t>(y) << 16);
}

// collect_row_extremes :676-715
void row_extremes(const bdo_frame& f, uint32_t root, int bx0, int bx1, int y0, int rows,
                  int kept, uint32_t* out) {
    const Params& p = f.p;
    for (int s = 0; s < kept; ++s) {
        const int y = y0 + (kept > 1 ? (s * (rows - 1)) / (kept - 1) : 0);
        const int n = static_cast<int>(f.row_count[y]);
        const uint32_t* row_runs = f.runs.data() + static_cast<size_t>(y) * p.row_cap;
        int lo = 0, hi = n - 1, first = n;
        while (lo <= hi) {
            const int mid = (lo + hi) >> 1;
            if (static_cast<int>(row_runs[mid] >> 16) >= bx0) {
                first = mid;
                hi = mid - 1;
            } else {
                lo = mid + 1;
            }
        }
        const uint32_t base = static_cast<uint32_t>(y * p.row_cap);
        int left = -1, right = -1;
        for (int k = first; k < n; ++k) {
            const int x0 = static_cast<int>(row_runs[k] & 0xffffu);
            const int x1 = static_cast<int>(row_runs[k] >> 16);
            if (x0 > bx1) break;
            if (f.label[base + static_cast<uint32_t>(k)] != root) continue;
            left = left < 0 ? x0 : std::min(left, x0);
            right = right < 0 ? x1 : std::max(right, x1);
        }
        out[2 * s] = left < 0 ? kNone : pack_point(left, y);
        out[2 * s + 1] = right < 0 ? kNone : pack_point(right, y);
    }
}

// The fit below is a template on its arithmetic type.  float is the
// restatement proper (the transcendental calls go through detmath.h, as on
// the GPU); double is the FP64 re-fit that the FP32 corners are measured
// against (bdo_refit64), with the C library's functions.
inline float fm_atan2(float y, float x) { return bdmath::atan2(y, x); }
inline double fm_atan2(double y, double x) { return std::atan2(y, x); }
inline void fm_sincos(float a, float* s, float* c) { bdmath::sincos(a, s, c); }
inline void fm_sincos(double a, double* s, double* c) {
    *s = std::sin(a);
    *c = std::cos(a);
}
inline float fm_hypot(float a, float b) { return bdmath::hypot(a, b); }
inline double fm_hypot(double a, double b) { return std::hypot(a, b); }
inline float two_pi(float) { return 6.28318530718f; }
inline double two_pi(double) { return 6.283185307179586; }

// hull_to_quad :736-831
template <typename T>
bool hull_to_quad(const uint32_t* hull, int count, T quad[4][2]) {
    if (count < 4 || count > kMaxHullVertices) return false;
    T vx[kMaxHullVertices];
    T vy[kMaxHullVertices];
    for (int i = 0; i < count; ++i) {
        vx[i] = static_cast<T>(hull[i] & 0xffffu);
        vy[i] = static_cast<T>(hull[i] >> 16);
    }
    while (count > 4) {
        int best = -1;
        T best_area = FLT_MAX;
        for (int i = 0; i < count; ++i) {
            const int prev = (i + count - 1) % count;
            const int next = (i + 1) % count;
            const T ax = vx[i] - vx[prev];
            const T ay = vy[i] - vy[prev];
            const T bx = vx[next] - vx[i];
            const T by = vy[next] - vy[i];
            const T area = std::fabs(ax * by - ay * bx) * 0.5f;
            if (area < best_area) {
                best_area = area;
                best = i;
            }
        }
        if (best < 0) return false;
        for (int i = best; i + 1 < count; ++i) {
            vx[i] = vx[i + 1];
            vy[i] = vy[i + 1];
        }
        --count;
    }
    T area2 = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        area2 += vx[i] * vy[j] - vx[j] * vy[i];
    }
    if (std::fabs(area2) < 24.0f) return false;
    if (area2 < 0.0f) {
        for (int i = 0; i < 2; ++i) {
            const T tx = vx[i + 1], ty = vy[i + 1];
            vx[i + 1] = vx[3 - i];
            vy[i + 1] = vy[3 - i];
            vx[3 - i] = tx;
            vy[3 - i] = ty;
        }
    }
    T min_side = FLT_MAX, max_side = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        const T ex = vx[j] - vx[i];
        const T ey = vy[j] - vy[i];
        const T len = std::sqrt(ex * ex + ey * ey);
        if (len < 4.0f) return false;
        min_side = std::fmin(min_side, len);
        max_side = std::fmax(max_side, len);
        const int pi = (i + 3) & 3;
        const T ax = vx[i] - vx[pi];
        const T ay = vy[i] - vy[pi];
        const T bx = vx[j] - vx[i];
        const T by = vy[j] - vy[i];
        if (ax * by - ay * bx <= 0.0f) return false;
        const T dot = ax * bx + ay * by;
        const T n1 = std::sqrt(ax * ax + ay * ay);
        const T n2 = std::sqrt(bx * bx + by * by);
        if (n1 < 1e-3f || n2 < 1e-3f) return false;
        if (std::fabs(dot / (n1 * n2)) > 0.97f) return false;
    }
    if (max_side > 12.0f * min_side) return false;
    const T cx = 0.25f * (vx[0] + vx[1] + vx[2] + vx[3]);
    const T cy = 0.25f * (vy[0] + vy[1] + vy[2] + vy[3]);
    for (int i = 0; i < 4; ++i) {
        const T dx = vx[i] - cx;
        const T dy = vy[i] - cy;
        const T len = std::sqrt(dx * dx + dy * dy);
        if (len > 1e-3f) {
            vx[i] += dx / len * 0.65f;
            vy[i] += dy / len * 0.65f;
        }
    }
    for (int i = 0; i < 4; ++i) {
        quad[i][0] = vx[i];
        quad[i][1] = vy[i];
    }
    return true;
}

// sample_bilinear :833-849
template <typename T>
T sample_bilinear(const uint8_t* image, int width, int height, int stride, T x, T y) {
    if (!(x >= 0.0f && y >= 0.0f && x < static_cast<T>(width - 1) &&
          y < static_cast<T>(height - 1))) {
        return -1.0f;
    }
    const int ix = static_cast<int>(x);
    const int iy = static_cast<int>(y);
    const T fx = x - static_cast<T>(ix);
    const T fy = y - static_cast<T>(iy);
    const uint8_t* q = image + static_cast<size_t>(iy) * stride + ix;
    const T a = q[0];
    const T b = q[1];
    const T c = q[stride];
    const T d = q[stride + 1];
    return (a * (1.0f - fx) + b * fx) * (1.0f - fy) + (c * (1.0f - fx) + d * fx) * fy;
}

// intersect_lines :851-859
template <typename T>
bool intersect_lines(const T li[4], const T lj[4], T* x, T* y) {
    const T det = li[2] * lj[3] - li[3] * lj[2];
    if (std::fabs(det) < 0.2f) return false;
    const T di = li[2] * li[0] + li[3] * li[1];
    const T dj = lj[2] * lj[0] + lj[3] * lj[1];
    *x = (di * lj[3] - li[3] * dj) / det;
    *y = (li[2] * dj - di * lj[2]) / det;
    return true;
}

// directional_rise :865-874
template <typename T>
T directional_rise(const uint8_t* image, int width, int height, int stride, T x, T y, T dx,
                   T dy) {
    const T ahead = sample_bilinear(image, width, height, stride, x + dx * 0.7f, y + dy * 0.7f);
    const T behind = sample_bilinear(image, width, height, stride, x - dx * 0.7f, y - dy * 0.7f);
    if (ahead < 0.0f || behind < 0.0f) return 0.0f;
    return ahead - behind;
}

// Sum of 32 lane values in the order a warp's __shfl_down_sync tree with
// offsets 16, 8, 4, 2, 1 leaves in lane 0.
template <typename T>
T warp_tree_sum(const T* v) {
    T a[32];
    for (int l = 0; l < 32; ++l) a[l] = v[l];
    for (int off = 16; off > 0; off >>= 1) {
        for (int l = 0; l < off; ++l) a[l] = a[l] + a[l + off];
    }
    return a[0];
}

// fit_edge_line_warp :881-1016, one lane per position along the edge.
template <typename T>
bool fit_edge_line(const T quad[4][2], int edge, const uint8_t* image, const Params& p, int dim,
                   bool first_pass, T line[4]) {
    const int width = p.width, height = p.height, stride = p.stride;
    const int b = (edge + 1) & 3;
    const T ax = quad[edge][0], ay = quad[edge][1];
    const T bx = quad[b][0], by = quad[b][1];
    const T ex = bx - ax;
    const T ey = by - ay;
    const T len = std::sqrt(ex * ex + ey * ey);
    if (len < 8.0f) return false;
    const T nx = ey / len;
    const T ny = -ex / len;
    const T cell = len / static_cast<T>(dim);
    const T range = first_pass ? std::fmin(std::fmax(1.15f * cell, 1.5f), 2.5f * cell)
                                   : std::fmin(std::fmax(0.30f * cell, 0.8f), 2.0f);
    const int half =
        std::min(std::max(2, static_cast<int>(std::ceil(range / 0.75f))), kFitProbeHalf);
    const int probes = 2 * half + 1;
    const T step = range / static_cast<T>(half);
    const int samples = std::min(std::max(static_cast<int>(len / 6.0f), 8), 16);

    T vmx[32] = {}, vmy[32] = {}, vmxx[32] = {}, vmxy[32] = {}, vmyy[32] = {};
    int vused[32] = {};
    for (int lane = 0; lane < samples; ++lane) {
        const T alpha = static_cast<T>(lane + 1) / static_cast<T>(samples + 1);
        const T px = ax + alpha * ex;
        const T py = ay + alpha * ey;
        T mags[kFitProbeHalf * 2 + 1];
        T best_mag = 0.0f;
        int best = -1;
        for (int i = 0; i < probes; ++i) {
            const T t = step * static_cast<T>(i - half);
            const T mag =
                directional_rise(image, width, height, stride, px + nx * t, py + ny * t, nx, ny);
            mags[i] = mag;
            if (mag > best_mag) {
                best_mag = mag;
                best = i;
            }
        }
        if (first_pass && best > 2) {
            const T accept = 0.70f * best_mag;
            for (int i = 1; i + 1 < best; ++i) {
                if (mags[i] < accept || mags[i] < mags[i - 1] || mags[i] < mags[i + 1]) continue;
                T valley = FLT_MAX;
                for (int k = i + 1; k < best; ++k) valley = std::fmin(valley, mags[k]);
                if (valley < 0.5f * mags[i]) {
                    best = i;
                    best_mag = mags[i];
                    break;
                }
            }
        }
        if (best >= 0 && best_mag >= 6.0f) {
            T t = step * static_cast<T>(best - half);
            if (best > 0 && best < probes - 1) {
                const T m0 = directional_rise(image, width, height, stride, px + nx * (t - step),
                                              py + ny * (t - step), nx, ny);
                const T m2 = directional_rise(image, width, height, stride, px + nx * (t + step),
                                              py + ny * (t + step), nx, ny);
                const T den = m0 - 2.0f * best_mag + m2;
                if (den < -1e-3f) {
                    t += std::fmin(std::fmax(0.5f * (m0 - m2) / den, -0.5f), 0.5f) * step;
                }
            }
            const T x = px + nx * t;
            const T y = py + ny * t;
            vmx[lane] = x;
            vmy[lane] = y;
            vmxx[lane] = x * x;
            vmxy[lane] = x * y;
            vmyy[lane] = y * y;
            vused[lane] = 1;
        }
    }
    const T mx = warp_tree_sum(vmx), my = warp_tree_sum(vmy);
    const T mxx = warp_tree_sum(vmxx), mxy = warp_tree_sum(vmxy), myy = warp_tree_sum(vmyy);
    const int used = warp_tree_sum(vused);
    if (used < 4) return false;
    const T inv = 1.0f / static_cast<T>(used);
    const T cx = mx * inv;
    const T cy = my * inv;
    const T cxx = mxx * inv - cx * cx;
    const T cxy = mxy * inv - cx * cy;
    const T cyy = myy * inv - cy * cy;
    const T theta = 0.5f * fm_atan2(2.0f * cxy, cxx - cyy);
    T s, c;
    fm_sincos(theta, &s, &c);
    line[0] = cx;
    line[1] = cy;
    line[2] = -s;
    line[3] = c;
    return true;
}

// apply_refined_lines :1021-1076
template <typename T>
T apply_refined_lines(T quad[4][2], const T lines[4][4], const int have[4]) {
    int line_count = 0;
    for (int i = 0; i < 4; ++i) line_count += have[i] ? 1 : 0;
    if (line_count < 3) return 0.0f;
    T refined[4][2];
    for (int i = 0; i < 4; ++i) {
        refined[i][0] = quad[i][0];
        refined[i][1] = quad[i][1];
    }
    T extent = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        extent = std::fmax(extent, fm_hypot(quad[j][0] - quad[i][0], quad[j][1] - quad[i][1]));
    }
    const T max_shift = std::fmin(std::fmax(0.15f * extent, 4.0f), 16.0f);
    T moved = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        if (!have[i] || !have[j]) continue;
        T x, y;
        if (!intersect_lines(lines[i], lines[j], &x, &y)) continue;
        const int corner = j;
        const T dx = x - quad[corner][0];
        const T dy = y - quad[corner][1];
        if (dx * dx + dy * dy > max_shift * max_shift) continue;
        refined[corner][0] = x;
        refined[corner][1] = y;
        moved = std::fmax(moved, std::sqrt(dx * dx + dy * dy));
    }
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        if (fm_hypot(refined[j][0] - refined[i][0], refined[j][1] - refined[i][1]) < 3.0f) {
            return 0.0f;
        }
    }
    T area2 = 0.0f;
    for (int i = 0; i < 4; ++i) {
        const int j = (i + 1) & 3;
        area2 += refined[i][0] * refined[j][1] - refined[j][0] * refined[i][1];
    }
    if (area2 <= 0.0f) return 0.0f;
    for (int i = 0; i < 4; ++i) {
        quad[i][0] = refined[i][0];
        quad[i][1] = refined[i][1];
    }
    return moved;
}

// The 32 probe directions of k_fit_quads :1139-1142.
template <typename T>
void probe_directions(T ux[kFitDirections], T uy[kFitDirections]) {
    for (int dir = 0; dir < kFitDirections; ++dir) {
        const T angle =
            two_pi(T()) * static_cast<T>(dir) / static_cast<T>(kFitDirections);
        fm_sincos(angle, &uy[dir], &ux[dir]);
    }
}

// k_fit_quads :1081-1241 for one candidate.  Returns true when the hull gave
// a quad (counts[3]); fills hull_out and out (8 floats each).
template <typename T>
bool fit_quad(const bdo_frame& f, const uint8_t* gray, uint32_t root, T* hull_out, T* out) {
    const Params& p = f.p;
    const int x0 = static_cast<int>(f.bbox[root * 4 + 0]);
    const int y0 = static_cast<int>(f.bbox[root * 4 + 1]);
    const int x1 = static_cast<int>(f.bbox[root * 4 + 2]);
    const int y1 = static_cast<int>(f.bbox[root * 4 + 3]);
    const int rows = y1 - y0 + 1;
    const int kept = std::min(rows, kMaxBoundaryRows);
    const int points = 2 * kept;
    std::vector<uint32_t> boundary(2 * kMaxBoundaryRows, kNone);
    row_extremes(f, root, x0, x1, y0, rows, kept, boundary.data());

    T ux[kFitDirections], uy[kFitDirections];
    probe_directions(ux, uy);
    uint32_t extreme[kFitDirections];
    for (int dir = 0; dir < kFitDirections; ++dir) {
        T best_dot = -FLT_MAX;
        uint32_t best_point = kNone;
        for (int i = 0; i < points; ++i) {
            const uint32_t q = boundary[i];
            if (q == kNone) continue;
            const T d =
                static_cast<T>(q & 0xffffu) * ux[dir] + static_cast<T>(q >> 16) * uy[dir];
            if (d > best_dot) {
                best_dot = d;
                best_point = q;
            }
        }
        extreme[dir] = best_point;
    }
    uint32_t hull[kFitDirections];
    int hc = 0;
    for (int i = 0; i < kFitDirections; ++i) {
        const uint32_t q = extreme[i];
        if (q == kNone) continue;
        if (hc > 0 && hull[hc - 1] == q) continue;
        hull[hc++] = q;
    }
    while (hc > 1 && hull[0] == hull[hc - 1]) --hc;

    T quad[4][2];
    if (!hull_to_quad(hull, hc, quad)) return false;
    for (int i = 0; i < 4; ++i) {
        hull_out[i * 2 + 0] = quad[i][0];
        hull_out[i * 2 + 1] = quad[i][1];
    }
    if (p.refine_edges) {
        for (int iteration = 0; iteration < kFitIterations; ++iteration) {
            T lines[4][4] = {};
            int have[4];
            for (int e = 0; e < 4; ++e) {
                have[e] = fit_edge_line(quad, e, gray, p, p.dim, iteration == 0, lines[e]) ? 1 : 0;
            }
            const T moved = apply_refined_lines(quad, lines, have);
            if (moved < 0.15f) break;
        }
    }
    for (int i = 0; i < 4; ++i) {
        out[i * 2 + 0] = quad[i][0];
        out[i * 2 + 1] = quad[i][1];
    }
    return true;
}

// --- 8. decode :1249-1537 ---------------------------------------------------

// homography_from_unit_quad :1249-1272
bool homography_from_unit_quad(const float quad[4][2], float h[9]) {
    const float x0 = quad[0][0], y0 = quad[0][1];
    const float x1 = quad[1][0], y1 = quad[1][1];
    const float x2 = quad[2][0], y2 = quad[2][1];
    const float x3 = quad[3][0], y3 = quad[3][1];
    const float dx1 = x1 - x2, dx2 = x3 - x2, dx3 = x0 - x1 + x2 - x3;
    const float dy1 = y1 - y2, dy2 = y3 - y2, dy3 = y0 - y1 + y2 - y3;
    const float det = dx1 * dy2 - dx2 * dy1;
    if (std::fabs(det) < 1e-9f) return false;
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

// match_code :1274-1289
int match_code(const uint64_t* codes, int count, uint64_t code, int max_hamming, int* out_hamming) {
    int best = max_hamming + 1;
    int best_id = -1;
    for (int i = 0; i < count; ++i) {
        const int d = popc64(codes[i] ^ code);
        if (d < best) {
            best = d;
            best_id = i;
            if (d == 0) break;
        }
    }
    if (best_id < 0) return -1;
    *out_hamming = best;
    return best_id;
}

// decode_quad :1291-1430 for one rotation.
bool decode_rotation(const uint8_t* gray, const Params& p, const float base_quad[4][2],
                     int rotation, DecodeOut* result) {
    const int dim = p.dim;
    float raw[64], diff[64], sharp[64];
    float corners[4][2];
    for (int k = 0; k < 4; ++k) {
        const int src = (rotation + k) & 3;
        corners[k][0] = base_quad[src][0];
        corners[k][1] = base_quad[src][1];
    }
    float h[9];
    if (!homography_from_unit_quad(corners, h)) return false;
    for (int cy = 0; cy < dim; ++cy) {
        for (int cx = 0; cx < dim; ++cx) {
            const float u = (cx + 0.5f) / static_cast<float>(dim);
            const float v = (cy + 0.5f) / static_cast<float>(dim);
            const float den = h[6] * u + h[7] * v + 1.0f;
            if (std::fabs(den) < 1e-9f) return false;
            const float x = (h[0] * u + h[1] * v + h[2]) / den;
            const float y = (h[3] * u + h[4] * v + h[5]) / den;
            const float value = sample_bilinear(gray, p.width, p.height, p.stride, x - 0.0f, y - 0.0f);
            if (value < 0.0f) return false;
            raw[cy * dim + cx] = value;
        }
    }
    float mn = 255.0f, mx = 0.0f;
    for (int i = 0; i < dim * dim; ++i) {
        mn = std::fmin(mn, raw[i]);
        mx = std::fmax(mx, raw[i]);
    }
    if (mx - mn < 10.0f) return false;
    const float thresh = 0.5f * (mn + mx);
    for (int cy = 0; cy < dim; ++cy) {
        for (int cx = 0; cx < dim; ++cx) {
            if (cx == 0 || cy == 0 || cx == dim - 1 || cy == dim - 1) {
                if (raw[cy * dim + cx] >= thresh) return false;
            }
        }
    }
    for (int i = 0; i < dim * dim; ++i) diff[i] = raw[i] - thresh;
    for (int i = 0; i < dim * dim; ++i) sharp[i] = diff[i];
    const int lo = 1, hi = dim - 2;
    for (int cy = lo; cy <= hi; ++cy) {
        for (int cx = lo; cx <= hi; ++cx) {
            const int i = cy * dim + cx;
            const float c = diff[i];
            const float lap = 4.0f * c - diff[i - dim] - diff[i + dim] - diff[i - 1] - diff[i + 1];
            sharp[i] = c + p.sharpening * lap;
        }
    }
    uint64_t code = 0;
    float white_sum = 0.0f, black_sum = 0.0f;
    int white_count = 0, black_count = 0;
    for (int cy = lo; cy <= hi; ++cy) {
        for (int cx = lo; cx <= hi; ++cx) {
            const float d = sharp[cy * dim + cx];
            code = (code << 1) | (d > 0.0f ? 1ull : 0ull);
            if (d > 0.0f) {
                white_sum += d;
                ++white_count;
            } else {
                black_sum -= d;
                ++black_count;
            }
        }
    }
    int hamming = 0;
    const int id = match_code(p.codes, p.code_count, code, p.max_hamming, &hamming);
    if (id < 0) return false;
    const float white_avg = white_sum / static_cast<float>(std::max(white_count, 1));
    const float black_avg = black_sum / static_cast<float>(std::max(black_count, 1));
    const float margin = std::fmin(white_avg, black_avg);
    if (margin < p.min_margin) return false;
    result->id = id;
    result->hamming = hamming;
    result->margin = margin;
    for (int k = 0; k < 4; ++k) {
        result->corners[k * 2 + 0] = corners[k][0];
        result->corners[k * 2 + 1] = corners[k][1];
    }
    return true;
}

// k_decode_quads :1438-1537 selection for one candidate: the refined quad's
// four rotations first, the hull's only when none of those decodes.
bool decode_candidate(const uint8_t* gray, const Params& p, const float* q, const float* hq,
                      DecodeOut* out) {
    if (q[0] != q[0]) return false;
    float quads[2][4][2];
    for (int i = 0; i < 4; ++i) {
        quads[0][i][0] = q[i * 2 + 0];
        quads[0][i][1] = q[i * 2 + 1];
        quads[1][i][0] = hq[i * 2 + 0];
        quads[1][i][1] = hq[i * 2 + 1];
    }
    DecodeOut results[8];
    bool ok[8];
    for (int lane = 0; lane < 8; ++lane) {
        ok[lane] = decode_rotation(gray, p, quads[lane >> 2], lane & 3, &results[lane]);
    }
    int best = -1;
    float best_score = -1.0f;
    for (int variant = 0; variant < 2 && best < 0; ++variant) {
        for (int rotation = 0; rotation < 4; ++rotation) {
            const int r = variant * 4 + rotation;
            if (!ok[r]) continue;
            const float score =
                static_cast<float>(4 - results[r].hamming) * 1000.0f + results[r].margin;
            if (score > best_score) {
                best_score = score;
                best = r;
            }
        }
    }
    if (best < 0) return false;
    *out = results[best];
    return true;
}

// --- 9. finalize :1542-1601 and the host homography :1739-1774 -------------

template <typename In, typename Out>
void fill_homography(const In corners[8], Out H[9]) {
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
    if (std::fabs(det) > 1e-12) {
        g = (dx3 * dy2 - dx2 * dy3) / det;
        h = (dx1 * dy3 - dx3 * dy1) / det;
    }
    const double a = x1 - x0 + g * x1;
    const double b = x3 - x0 + h * x3;
    const double d = y1 - y0 + g * y1;
    const double e = y3 - y0 + h * y3;
    const double w = g + h + 2.0;
    const double inv = (std::fabs(w) > 1e-12) ? 1.0 / w : 0.0;
    H[0] = static_cast<Out>(a * inv);
    H[1] = static_cast<Out>(b * inv);
    H[2] = static_cast<Out>((a + b + 2.0 * x0) * inv);
    H[3] = static_cast<Out>(d * inv);
    H[4] = static_cast<Out>(e * inv);
    H[5] = static_cast<Out>((d + e + 2.0 * y0) * inv);
    H[6] = static_cast<Out>(g * inv);
    H[7] = static_cast<Out>(h * inv);
    H[8] = static_cast<Out>(w * inv);
}

void finalize(bdo_frame& f) {
    const Params& p = f.p;
    // Detection slots in candidate order, capped at max_detections.
    std::vector<bd_detection> slots;
    uint32_t decoded = 0;
    for (size_t ci = 0; ci < f.decodes.size(); ++ci) {
        const DecodeOut& r = f.decodes[ci];
        if (r.id < 0) continue;
        ++decoded;
        if (slots.size() >= static_cast<size_t>(p.max_detections)) continue;
        bd_detection d;
        std::memset(&d, 0, sizeof(d));
        d.id = r.id;
        d.hamming = r.hamming;
        d.decision_margin = r.margin;
        for (int k = 0; k < 8; ++k) d.corners[k] = r.corners[k];
        d.reserved = 0;
        slots.push_back(d);
    }
    (void)decoded;
    std::vector<bd_detection> out;
    for (const bd_detection& d : slots) {
        float side = 0.0f, cx = 0.0f, cy = 0.0f;
        for (int k = 0; k < 4; ++k) {
            const int j = (k + 1) & 3;
            side += bdmath::hypot(d.corners[j * 2] - d.corners[k * 2],
                                  d.corners[j * 2 + 1] - d.corners[k * 2 + 1]);
            cx += d.corners[k * 2];
            cy += d.corners[k * 2 + 1];
        }
        side *= 0.25f;
        cx *= 0.25f;
        cy *= 0.25f;
        int duplicate = -1;
        for (size_t k = 0; k < out.size(); ++k) {
            if (out[k].id != d.id) continue;
            float ocx = 0.0f, ocy = 0.0f;
            for (int c = 0; c < 4; ++c) {
                ocx += out[k].corners[c * 2];
                ocy += out[k].corners[c * 2 + 1];
            }
            ocx *= 0.25f;
            ocy *= 0.25f;
            const float limit = 0.35f * side;
            if (std::fabs(ocx - cx) < limit && std::fabs(ocy - cy) < limit) {
                duplicate = static_cast<int>(k);
                break;
            }
        }
        if (duplicate >= 0) {
            if (d.decision_margin > out[duplicate].decision_margin) out[duplicate] = d;
        } else if (out.size() < static_cast<size_t>(p.max_detections)) {
            out.push_back(d);
        }
    }
    std::stable_sort(out.begin(), out.end(),
                     [](const bd_detection& a, const bd_detection& b) { return a.id < b.id; });
    for (bd_detection& d : out) fill_homography(d.corners, d.homography);
    f.counts[1] = static_cast<uint32_t>(out.size());
    f.detections = out;
}

void run_pipeline(const uint8_t* gray, bdo_frame& f) {
    std::memset(f.counts, 0, sizeof(f.counts));
    tile_stats(gray, f);
    tile_reference(f);
    tile_threshold(f);
    row_roi(f);
    binarize(gray, f);
    find_runs(f);
    merge_runs(f);
    region_stats(f);
    collect_candidates(f);
    const int mc = f.p.max_candidates;
    f.hull_quads.assign(static_cast<size_t>(mc) * 8, bdmath::quiet_nan());
    f.quads.assign(static_cast<size_t>(mc) * 8, bdmath::quiet_nan());
    f.decodes.assign(f.candidates.size(), DecodeOut{-1, 0, 0.0f, {}});
    for (size_t ci = 0; ci < f.candidates.size(); ++ci) {
        if (fit_quad(f, gray, f.candidates[ci], &f.hull_quads[ci * 8], &f.quads[ci * 8])) {
            f.counts[3] += 1;
        }
    }
    for (size_t ci = 0; ci < f.candidates.size(); ++ci) {
        DecodeOut r;
        if (decode_candidate(gray, f.p, &f.quads[ci * 8], &f.hull_quads[ci * 8], &r)) {
            f.decodes[ci] = r;
        }
    }
    finalize(f);
}

template <typename T>
int64_t copy_out(const std::vector<T>& v, void* dst, int64_t dst_bytes) {
    const int64_t bytes = static_cast<int64_t>(v.size() * sizeof(T));
    if (dst && dst_bytes > 0) std::memcpy(dst, v.data(), static_cast<size_t>(std::min(bytes, dst_bytes)));
    return bytes;
}

int64_t copy_raw(const void* src, int64_t bytes, void* dst, int64_t dst_bytes) {
    if (dst && dst_bytes > 0) std::memcpy(dst, src, static_cast<size_t>(std::min(bytes, dst_bytes)));
    return bytes;
}

}  // namespace

extern "C" {

bdo_frame* bdo_run(const uint8_t* gray, int32_t width, int32_t height, int32_t stride,
                   int32_t family, const bd_config* config) {
    if (!gray || family < 0 || family > 1 || width < 16 || height < 16 || width > BD_MAX_WIDTH ||
        height > BD_MAX_HEIGHT || stride < width) {
        return nullptr;
    }
    bdo_frame* f = new bdo_frame();
    f->p = resolve(family, width, height, stride, config);
    run_pipeline(gray, *f);
    return f;
}

void bdo_free(bdo_frame* frame) { delete frame; }

int32_t bdo_detections(const bdo_frame* f, bd_detection* out, int32_t capacity) {
    const int found = static_cast<int>(f->detections.size());
    const int written = std::min(found, std::max(capacity, 0));
    if (out && written > 0) {
        std::memcpy(out, f->detections.data(), static_cast<size_t>(written) * sizeof(bd_detection));
    }
    return found;
}

void bdo_counts(const bdo_frame* f, uint32_t counts[5]) {
    std::memcpy(counts, f->counts, sizeof(f->counts));
}

void bdo_geometry(const bdo_frame* f, int32_t out[9]) {
    out[0] = f->p.tile_w;
    out[1] = f->p.tile_h;
    out[2] = f->p.words;
    out[3] = f->p.row_cap;
    out[4] = f->p.max_candidates;
    out[5] = f->p.max_detections;
    out[6] = f->p.dim;
    out[7] = f->p.max_hamming;
    out[8] = static_cast<int32_t>(f->candidates.size());
}

int64_t bdo_stage(const bdo_frame* f, const char* name, void* dst, int64_t dst_bytes) {
    const std::string n(name ? name : "");
    if (n == "tile_min") return copy_out(f->tile_min, dst, dst_bytes);
    if (n == "tile_max") return copy_out(f->tile_max, dst, dst_bytes);
    if (n == "tile_mean") return copy_out(f->tile_mean, dst, dst_bytes);
    if (n == "thresh") return copy_out(f->thresh, dst, dst_bytes);
    if (n == "active") return copy_out(f->active, dst, dst_bytes);
    if (n == "span_hist") return copy_raw(f->span_hist, sizeof(f->span_hist), dst, dst_bytes);
    if (n == "mean_hist") return copy_raw(f->mean_hist, sizeof(f->mean_hist), dst, dst_bytes);
    if (n == "ref") return copy_raw(f->ref, sizeof(f->ref), dst, dst_bytes);
    if (n == "row_active") return copy_out(f->row_active, dst, dst_bytes);
    if (n == "row_start") return copy_out(f->row_start, dst, dst_bytes);
    if (n == "row_end") return copy_out(f->row_end, dst, dst_bytes);
    if (n == "bits") return copy_out(f->bits, dst, dst_bytes);
    if (n == "row_count") return copy_out(f->row_count, dst, dst_bytes);
    if (n == "runs") return copy_out(f->runs, dst, dst_bytes);
    if (n == "label") return copy_out(f->label, dst, dst_bytes);
    if (n == "area") return copy_out(f->area, dst, dst_bytes);
    if (n == "bbox") return copy_out(f->bbox, dst, dst_bytes);
    if (n == "candidates") return copy_out(f->candidates, dst, dst_bytes);
    if (n == "hull_quads") return copy_out(f->hull_quads, dst, dst_bytes);
    if (n == "quads") return copy_out(f->quads, dst, dst_bytes);
    if (n == "decodes") return copy_out(f->decodes, dst, dst_bytes);
    return -1;
}

int32_t bdo_detect_many(int32_t frames, const uint8_t* const* grays, const int32_t* widths,
                        const int32_t* heights, const int32_t* strides,
                        const uint32_t* family_masks, const bd_config* config, int32_t threads,
                        bd_detection* out, int32_t max_detections, int32_t* counts) {
    if (frames < 0 || !grays || !widths || !heights || !strides || !family_masks || !out ||
        !counts || max_detections < 1) {
        return -1;
    }
    // Work units are (frame, family) pairs, so a few frames still keep every
    // thread busy.
    std::atomic<int32_t> next{0};
    const int nthreads = std::max(1, threads);
    auto worker = [&]() {
        for (;;) {
            const int32_t unit = next.fetch_add(1);
            if (unit >= 2 * frames) return;
            const int32_t i = unit >> 1;
            const int fam = unit & 1;
            int32_t* count = &counts[i * 2 + fam];
            bd_detection* dst = out + (static_cast<size_t>(i) * 2 + fam) * max_detections;
            if (!(family_masks[i] & (1u << fam))) {
                *count = -1;
                continue;
            }
            bdo_frame* f = bdo_run(grays[i], widths[i], heights[i], strides[i], fam, config);
            if (!f) {
                *count = -1;
                continue;
            }
            *count = bdo_detections(f, dst, max_detections);
            bdo_free(f);
        }
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto& t : pool) t.join();
    return 0;
}

int32_t bdo_refit64(const bdo_frame* f, const uint8_t* gray, double* hull_out, double* quads_out) {
    const int n = static_cast<int>(f->candidates.size());
    const double nan = std::numeric_limits<double>::quiet_NaN();
    for (int ci = 0; ci < n; ++ci) {
        double* hq = hull_out + static_cast<size_t>(ci) * 8;
        double* q = quads_out + static_cast<size_t>(ci) * 8;
        for (int k = 0; k < 8; ++k) hq[k] = q[k] = nan;
        fit_quad(*f, gray, f->candidates[ci], hq, q);
    }
    return n;
}

void bdo_homography64(const double corners[8], double H[9]) { fill_homography(corners, H); }

float bdo_sinf(float x) { return bdmath::sin(x); }
float bdo_cosf(float x) { return bdmath::cos(x); }
float bdo_atan2f(float y, float x) { return bdmath::atan2(y, x); }

}  // extern "C"
