// Synthetic frames with exact ground truth, for the tests and the benchmark.
//
// Three generators:
//  * bds_make_pose / bds_render_tag: the reference's test renderer
//    conventions (reference detector/tests/test_support.hpp:46-137): tag
//    frame [-1, 1]^2 = black square, row-major MSB-first data cells, 2x2
//    supersampling, white background, min-compositing.  The reference's
//    known-answer tests are defined on frames drawn this way.
//  * bds_ref_scenes: the reference's benchmark scene set
//    (detector/bench/scenes.hpp:64-206: mix32 stream, 8 tag36h11 ids on a
//    jittered 4x2 grid, decoys on scenes s % 8 == 3, uniform noise in
//    [-3, 3]).  The steps have to be the same to give the same pixels; the
//    tests compare SHA-256 hashes of these frames with frames written by the
//    reference's own scene exporter.
//  * bds_render_scene: this project's seeded generator for the five
//    workload scene sets (gradient background, Gaussian-like noise, both
//    families, perspective tilt, blur, decoys, glyph clutter).  It uses only
//    integer arithmetic and IEEE double +, -, *, /, sqrt (own sin/cos), so a
//    seed gives the same frame on x86 and Arm.
//
// Ground-truth corners use the reference's pixel-index convention
// (scenes.hpp:40-58): pixel i covers [i, i+1) and is sampled at i + 0.5, so a
// continuous edge at x appears at index x - 0.5.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

#include "families_data.inc"

const uint64_t kCodewords36h11[BD_CODEWORDS_36H11_COUNT] = {BD_CODEWORDS_36H11};
const uint64_t kCodewords16h5[BD_CODEWORDS_16H5_COUNT] = {BD_CODEWORDS_16H5};

struct FamilyInfo {
    int bits;
    int count;
    const uint64_t* codes;
};

const FamilyInfo kFam[2] = {{6, 587, kCodewords36h11}, {4, 30, kCodewords16h5}};

struct Mat3 {
    double v[9];
    void project(double x, double y, double* ox, double* oy) const {
        const double w = v[6] * x + v[7] * y + v[8];
        *ox = (v[0] * x + v[1] * y + v[2]) / w;
        *oy = (v[3] * x + v[4] * y + v[5]) / w;
    }
    Mat3 inverse() const {
        const double a = v[0], b = v[1], c = v[2];
        const double d = v[3], e = v[4], f = v[5];
        const double g = v[6], h = v[7], i = v[8];
        const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
        const double inv = 1.0 / det;
        Mat3 o{};
        o.v[0] = (e * i - f * h) * inv;
        o.v[1] = (c * h - b * i) * inv;
        o.v[2] = (b * f - c * e) * inv;
        o.v[3] = (f * g - d * i) * inv;
        o.v[4] = (a * i - c * g) * inv;
        o.v[5] = (c * d - a * f) * inv;
        o.v[6] = (d * h - e * g) * inv;
        o.v[7] = (b * g - a * h) * inv;
        o.v[8] = (a * e - b * d) * inv;
        return o;
    }
};

int popcount64(uint64_t v) { return __builtin_popcountll(v); }

uint64_t rotate_code(uint64_t code, int bits) {
    const int n = bits * bits;
    uint64_t out = 0;
    for (int r = 0; r < bits; ++r) {
        for (int c = 0; c < bits; ++c) {
            const uint64_t bit = (code >> (n - 1 - (r * bits + c))) & 1ull;
            out |= bit << (n - 1 - (c * bits + (bits - 1 - r)));
        }
    }
    return out;
}

// ---------------------------------------------------------------------------
// Reference test renderer conventions (test_support.hpp:46-137).
// ---------------------------------------------------------------------------
Mat3 make_pose(double cx, double cy, double size_px, double angle, double perspective) {
    const double c = std::cos(angle);
    const double s = std::sin(angle);
    const double h = 0.5 * size_px;
    Mat3 m{};
    m.v[0] = c * h;
    m.v[1] = -s * h;
    m.v[2] = cx;
    m.v[3] = s * h;
    m.v[4] = c * h;
    m.v[5] = cy;
    m.v[6] = perspective * c;
    m.v[7] = -perspective * s;
    m.v[8] = 1.0;
    return m;
}

// Draws one tag into a width x height patch initialised to 255.
void render_patch(int family, uint64_t code, int width, int height, const Mat3& pose, int ss,
                  bool flip_one_bit, uint8_t* image) {
    const int bits = kFam[family].bits;
    const int border = 1;
    const int dim = bits + 2 * border;
    const Mat3 inv = pose.inverse();
    ss = std::max(1, ss);
    for (int py = 0; py < height; ++py) {
        for (int px = 0; px < width; ++px) {
            int accum = 0;
            for (int sy = 0; sy < ss; ++sy) {
                for (int sx = 0; sx < ss; ++sx) {
                    const double ix = px + (sx + 0.5) / ss;
                    const double iy = py + (sy + 0.5) / ss;
                    double tx, ty;
                    inv.project(ix, iy, &tx, &ty);
                    if (tx < -1.0 || tx > 1.0 || ty < -1.0 || ty > 1.0) {
                        accum += 255;
                        continue;
                    }
                    const int cx = std::min(dim - 1, std::max(0, static_cast<int>((tx + 1.0) * 0.5 * dim)));
                    const int cy = std::min(dim - 1, std::max(0, static_cast<int>((ty + 1.0) * 0.5 * dim)));
                    if (cx == 0 || cy == 0 || cx == dim - 1 || cy == dim - 1) continue;
                    const int pos = (cy - border) * bits + (cx - border);
                    uint64_t cell = (code >> (bits * bits - 1 - pos)) & 1ull;
                    if (flip_one_bit && pos == 0) cell ^= 1ull;
                    accum += cell ? 255 : 0;
                }
            }
            image[static_cast<size_t>(py) * width + px] = static_cast<uint8_t>(accum / (ss * ss));
        }
    }
}

// ---------------------------------------------------------------------------
// Reference benchmark scenes (scenes.hpp:40-206).
// ---------------------------------------------------------------------------
uint32_t mix32(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

double next_unit(uint32_t& state) {
    state = mix32(state + 0x9e3779b9u);
    return (state >> 8) * (1.0 / 16777216.0);
}

void ref_square(const Mat3& pose, double out[4][2]) {
    static const double kUnit[4][2] = {{-1.0, -1.0}, {1.0, -1.0}, {1.0, 1.0}, {-1.0, 1.0}};
    for (int i = 0; i < 4; ++i) {
        pose.project(kUnit[i][0], kUnit[i][1], &out[i][0], &out[i][1]);
        out[i][0] -= 0.5;
        out[i][1] -= 0.5;
    }
}

void ref_render_into(std::vector<uint8_t>& image, int width, int height, int family, uint64_t code,
                     const Mat3& pose) {
    double c[4][2];
    ref_square(pose, c);
    double min_x = c[0][0], max_x = c[0][0], min_y = c[0][1], max_y = c[0][1];
    for (int i = 1; i < 4; ++i) {
        min_x = std::min(min_x, c[i][0]);
        max_x = std::max(max_x, c[i][0]);
        min_y = std::min(min_y, c[i][1]);
        max_y = std::max(max_y, c[i][1]);
    }
    const int margin = 4;
    const int x0 = std::max(0, static_cast<int>(std::floor(min_x)) - margin);
    const int y0 = std::max(0, static_cast<int>(std::floor(min_y)) - margin);
    const int x1 = std::min(width - 1, static_cast<int>(std::ceil(max_x)) + margin);
    const int y1 = std::min(height - 1, static_cast<int>(std::ceil(max_y)) + margin);
    if (x1 < x0 || y1 < y0) return;
    const int rw = x1 - x0 + 1, rh = y1 - y0 + 1;
    Mat3 shifted = pose;
    shifted.v[2] -= x0;
    shifted.v[5] -= y0;
    std::vector<uint8_t> patch(static_cast<size_t>(rw) * rh, 255);
    render_patch(family, code, rw, rh, shifted, 2, false, patch.data());
    for (int y = 0; y < rh; ++y) {
        uint8_t* dst = image.data() + static_cast<size_t>(y0 + y) * width + x0;
        const uint8_t* src = patch.data() + static_cast<size_t>(y) * rw;
        for (int x = 0; x < rw; ++x) dst[x] = std::min(dst[x], src[x]);
    }
}

uint64_t ref_non_tag_code(uint32_t& rng, int family, int min_distance) {
    const int cells = kFam[family].bits * kFam[family].bits;
    const uint64_t mask = cells >= 64 ? ~0ull : ((1ull << cells) - 1ull);
    for (;;) {
        const uint64_t code = ((static_cast<uint64_t>(mix32(rng)) << 32) ^ mix32(rng)) & mask;
        int best = 1000;
        for (int i = 0; i < kFam[family].count; ++i) {
            uint64_t rotated = kFam[family].codes[i];
            for (int k = 0; k < 4; ++k) {
                best = std::min(best, popcount64(code ^ rotated));
                rotated = rotate_code(rotated, kFam[family].bits);
            }
        }
        if (best >= min_distance) return code;
    }
}

// ---------------------------------------------------------------------------
// Seeded workload generator.
// ---------------------------------------------------------------------------
uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ull;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ull;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebull;
    return x ^ (x >> 31);
}

struct Rng {
    uint64_t state;
    uint64_t next() {
        state += 0x9e3779b97f4a7c15ull;
        return splitmix64(state);
    }
    double unit() { return static_cast<double>(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double a, double b) { return a + (b - a) * unit(); }
    int range(int a, int b) { return a + static_cast<int>(next() % static_cast<uint64_t>(b - a + 1)); }
};

// sin/cos in double from +, -, *, /: reduce by pi/2 (two-part constant),
// then Taylor series to r^19 / r^20 on |r| <= pi/4.  Deterministic across
// hosts, unlike libm.
void dsincos(double x, double* s, double* c) {
    const double kPio2Hi = 1.5707963267341256e+00;
    const double kPio2Lo = 6.0771005065061922e-11;
    const double k = std::floor(x * 0.6366197723675814 + 0.5);
    const double r = (x - k * kPio2Hi) - k * kPio2Lo;
    const double r2 = r * r;
    double ts = r, tc = 1.0, term_s = r, term_c = 1.0;
    for (int n = 1; n <= 10; ++n) {
        term_s = -term_s * r2 / static_cast<double>((2 * n) * (2 * n + 1));
        term_c = -term_c * r2 / static_cast<double>((2 * n - 1) * (2 * n));
        ts += term_s;
        tc += term_c;
    }
    const int q = static_cast<int>(static_cast<int64_t>(k) & 3);
    if (q == 0) { *s = ts; *c = tc; }
    else if (q == 1) { *s = tc; *c = -ts; }
    else if (q == 2) { *s = -ts; *c = -tc; }
    else { *s = -tc; *c = ts; }
}

// A tag pose: in-plane rotation theta, out-of-plane tilt alpha about the
// in-plane axis at angle phi, seen by a pinhole camera with focal length
// f = 1000 px at distance f, centred at (cx, cy); side = black-square side
// in pixels at zero tilt.  Maps tag coordinates to pixels.
Mat3 tilted_pose(double cx, double cy, double side, double theta, double alpha, double phi) {
    double st, ct, sa, ca, sp, cp;
    dsincos(theta, &st, &ct);
    dsincos(alpha, &sa, &ca);
    dsincos(phi, &sp, &cp);
    // Rotation about unit axis (cp, sp, 0) by alpha (Rodrigues).
    const double ux = cp, uy = sp;
    const double one_c = 1.0 - ca;
    double Rt[9] = {ca + ux * ux * one_c, ux * uy * one_c, uy * sa,
                    uy * ux * one_c,      ca + uy * uy * one_c, -ux * sa,
                    -uy * sa,             ux * sa,              ca};
    const double Rz[9] = {ct, -st, 0.0, st, ct, 0.0, 0.0, 0.0, 1.0};
    double R[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j)
            R[i * 3 + j] = Rz[i * 3 + 0] * Rt[0 * 3 + j] + Rz[i * 3 + 1] * Rt[1 * 3 + j] +
                           Rz[i * 3 + 2] * Rt[2 * 3 + j];
    const double f = 1000.0, Z = 1000.0, hs = 0.5 * side;
    Mat3 m{};
    m.v[0] = (f * R[0] + cx * R[6]) * hs / Z;
    m.v[1] = (f * R[1] + cx * R[7]) * hs / Z;
    m.v[2] = cx;
    m.v[3] = (f * R[3] + cy * R[6]) * hs / Z;
    m.v[4] = (f * R[4] + cy * R[7]) * hs / Z;
    m.v[5] = cy;
    m.v[6] = R[6] * hs / Z;
    m.v[7] = R[7] * hs / Z;
    m.v[8] = 1.0;
    return m;
}

struct Box {
    double x0, y0, x1, y1;
};

bool overlaps(const Box& a, const Box& b) {
    return !(a.x1 < b.x0 || b.x1 < a.x0 || a.y1 < b.y0 || b.y1 < a.y0);
}

// Draws a tag (black square + data cells + one-cell white quiet zone) with
// S x S supersampling over its footprint; samples outside the quiet zone keep
// the background pixel.  Values: black 30, white 220.
void draw_tag(uint8_t* image, int width, int height, int family, uint64_t code, const Mat3& pose,
              const Box& box) {
    const int bits = kFam[family].bits;
    const int dim = bits + 2;                 // cells across the black square
    const double cell = 2.0 / dim;            // cell size in tag units
    const double outer = 1.0 + cell;          // quiet zone edge
    const Mat3 inv = pose.inverse();
    const int S = 4;
    const int x0 = std::max(0, static_cast<int>(std::floor(box.x0)));
    const int y0 = std::max(0, static_cast<int>(std::floor(box.y0)));
    const int x1 = std::min(width - 1, static_cast<int>(std::ceil(box.x1)));
    const int y1 = std::min(height - 1, static_cast<int>(std::ceil(box.y1)));
    for (int py = y0; py <= y1; ++py) {
        for (int px = x0; px <= x1; ++px) {
            uint8_t& dst = image[static_cast<size_t>(py) * width + px];
            int accum = 0;
            int inside = 0;
            for (int sy = 0; sy < S; ++sy) {
                for (int sx = 0; sx < S; ++sx) {
                    double tx, ty;
                    inv.project(px + (sx + 0.5) / S, py + (sy + 0.5) / S, &tx, &ty);
                    if (tx < -outer || tx > outer || ty < -outer || ty > outer) {
                        accum += dst;
                        continue;
                    }
                    ++inside;
                    if (tx < -1.0 || tx > 1.0 || ty < -1.0 || ty > 1.0) {
                        accum += 220;
                        continue;
                    }
                    const int cx = std::min(dim - 1, std::max(0, static_cast<int>((tx + 1.0) / cell)));
                    const int cy = std::min(dim - 1, std::max(0, static_cast<int>((ty + 1.0) / cell)));
                    if (cx == 0 || cy == 0 || cx == dim - 1 || cy == dim - 1) {
                        accum += 30;
                        continue;
                    }
                    const int pos = (cy - 1) * bits + (cx - 1);
                    accum += ((code >> (bits * bits - 1 - pos)) & 1ull) ? 220 : 30;
                }
            }
            if (inside) dst = static_cast<uint8_t>((accum + S * S / 2) / (S * S));
        }
    }
}

// Footprint (quiet-zone square) of a pose, in pixels.
Box footprint(const Mat3& pose, int family) {
    const double outer = 1.0 + 2.0 / (kFam[family].bits + 2);
    Box b{1e30, 1e30, -1e30, -1e30};
    const double u[4][2] = {{-outer, -outer}, {outer, -outer}, {outer, outer}, {-outer, outer}};
    for (int i = 0; i < 4; ++i) {
        double x, y;
        pose.project(u[i][0], u[i][1], &x, &y);
        b.x0 = std::min(b.x0, x);
        b.y0 = std::min(b.y0, y);
        b.x1 = std::max(b.x1, x);
        b.y1 = std::max(b.y1, y);
    }
    return b;
}

// A code in `family`'s layout at Hamming distance >= min_distance from every
// rotation of every codeword of that family.
uint64_t decoy_code(Rng& rng, int family, int min_distance) {
    const int cells = kFam[family].bits * kFam[family].bits;
    const uint64_t mask = (1ull << cells) - 1ull;
    for (;;) {
        const uint64_t code = rng.next() & mask;
        int best = 1000;
        for (int i = 0; i < kFam[family].count && best >= min_distance; ++i) {
            uint64_t rotated = kFam[family].codes[i];
            for (int k = 0; k < 4; ++k) {
                best = std::min(best, popcount64(code ^ rotated));
                rotated = rotate_code(rotated, kFam[family].bits);
            }
        }
        if (best >= min_distance) return code;
    }
}

struct Tag {
    int32_t family;
    int32_t id;
    double corners[8];
};

struct SceneSpec {
    double background = 128.0;
    double gradient = 20.0;
    double sigma = 4.0;
    int n36 = 8, n16 = 0;
    double side_min = 40.0, side_max = 120.0;
    double max_tilt = 0.7853981633974483;  // 45 degrees
    bool blur = false;
    int decoys = 0;
    int glyphs = 0;
    bool blank = false;
};

// Approximately normal deviate from one 64-bit hash: the sum of four
// 16-bit uniforms (Irwin-Hall, n = 4), scaled to unit variance.
double normal_from_hash(uint64_t h) {
    double s = 0.0;
    for (int k = 0; k < 4; ++k) s += static_cast<double>((h >> (16 * k)) & 0xffffu) * (1.0 / 65536.0);
    return (s - 2.0) * 1.7320508075688772;
}

int render_scene(const SceneSpec& spec, uint64_t seed, int width, int height, uint8_t* image,
                 Tag* tags, int max_tags) {
    Rng rng{splitmix64(seed)};
    // Background: level + linear gradient of +-gradient along a random direction.
    double gs, gc;
    dsincos(rng.uniform(0.0, 6.283185307179586), &gs, &gc);
    const double half_diag = 0.5 * std::sqrt(static_cast<double>(width) * width +
                                             static_cast<double>(height) * height);
    for (int y = 0; y < height; ++y) {
        for (int x = 0; x < width; ++x) {
            const double t = ((x - 0.5 * width) * gc + (y - 0.5 * height) * gs) / half_diag;
            double v = spec.background + spec.gradient * t;
            v = std::min(255.0, std::max(0.0, v));
            image[static_cast<size_t>(y) * width + x] = static_cast<uint8_t>(v + 0.5);
        }
    }
    int count = 0;
    std::vector<Box> placed;
    auto place = [&](int family, uint64_t code, int id, bool is_tag, double side_min,
                     double side_max) -> bool {
        for (int attempt = 0; attempt < 60; ++attempt) {
            const double side = rng.uniform(side_min, side_max);
            const double margin = 0.75 * side + 4.0;
            if (width <= 2 * margin || height <= 2 * margin) continue;
            const double cx = rng.uniform(margin, width - margin);
            const double cy = rng.uniform(margin, height - margin);
            const double theta = rng.uniform(0.0, 6.283185307179586);
            const double alpha = rng.uniform(0.0, spec.max_tilt);
            const double phi = rng.uniform(0.0, 3.141592653589793);
            const Mat3 pose = tilted_pose(cx, cy, side, theta, alpha, phi);
            Box b = footprint(pose, family);
            if (b.x0 < 2 || b.y0 < 2 || b.x1 > width - 3 || b.y1 > height - 3) continue;
            Box padded{b.x0 - 3, b.y0 - 3, b.x1 + 3, b.y1 + 3};
            bool clash = false;
            for (const Box& o : placed) clash = clash || overlaps(padded, o);
            if (clash) continue;
            placed.push_back(padded);
            draw_tag(image, width, height, family, code, pose, b);
            if (is_tag && count < max_tags) {
                Tag& t = tags[count++];
                t.family = family;
                t.id = id;
                static const double kUnit[4][2] = {{-1, -1}, {1, -1}, {1, 1}, {-1, 1}};
                for (int k = 0; k < 4; ++k) {
                    double x, y;
                    pose.project(kUnit[k][0], kUnit[k][1], &x, &y);
                    t.corners[2 * k] = x - 0.5;
                    t.corners[2 * k + 1] = y - 0.5;
                }
            }
            return true;
        }
        return false;
    };
    if (!spec.blank) {
        // Ids uniform without replacement within each family.
        std::vector<int> ids36(587), ids16(30);
        for (int i = 0; i < 587; ++i) ids36[i] = i;
        for (int i = 0; i < 30; ++i) ids16[i] = i;
        for (int i = 586; i > 0; --i) std::swap(ids36[i], ids36[rng.range(0, i)]);
        for (int i = 29; i > 0; --i) std::swap(ids16[i], ids16[rng.range(0, i)]);
        const int total = spec.n36 + spec.n16;
        for (int k = 0; k < total; ++k) {
            const int family = k < spec.n36 ? 0 : 1;
            const int id = family == 0 ? ids36[k % 587] : ids16[(k - spec.n36) % 30];
            place(family, kFam[family].codes[id], id, true, spec.side_min, spec.side_max);
        }
        for (int k = 0; k < spec.decoys; ++k) {
            place(0, decoy_code(rng, 0, 4), -1, false, std::max(spec.side_min, 40.0),
                  std::max(spec.side_min, 40.0) + 60.0);
        }
        // Glyph clutter: hollow rectangles and bars, each a tag-like
        // connected component that passes the candidate filter.
        for (int g = 0; g < spec.glyphs; ++g) {
            for (int attempt = 0; attempt < 8; ++attempt) {
                const int gw = rng.range(9, 18), gh = rng.range(9, 18);
                const int gx = rng.range(4, width - gw - 5), gy = rng.range(4, height - gh - 5);
                Box b{gx - 2.0, gy - 2.0, gx + gw + 2.0, gy + gh + 2.0};
                bool clash = false;
                for (const Box& o : placed) clash = clash || overlaps(b, o);
                if (clash) continue;
                placed.push_back(b);
                const int stroke = rng.range(2, 3);
                const int shape = rng.range(0, 2);
                for (int y = gy; y < gy + gh; ++y) {
                    for (int x = gx; x < gx + gw; ++x) {
                        const bool edge = x < gx + stroke || x >= gx + gw - stroke ||
                                          y < gy + stroke || y >= gy + gh - stroke;
                        const bool bar = shape == 2 && (y - gy) >= gh / 2 - 1 && (y - gy) <= gh / 2;
                        const bool open = shape == 1 && x >= gx + gw - stroke && y > gy + gh / 3 &&
                                          y < gy + 2 * gh / 3;
                        if ((edge && !open) || bar) image[static_cast<size_t>(y) * width + x] = 30;
                    }
                }
                break;
            }
        }
    }
    if (spec.blur) {
        // 3x3 binomial blur [1 2 1]^T [1 2 1] / 16, edges replicated.
        std::vector<uint8_t> src(image, image + static_cast<size_t>(width) * height);
        for (int y = 0; y < height; ++y) {
            const int ym = std::max(0, y - 1), yp = std::min(height - 1, y + 1);
            for (int x = 0; x < width; ++x) {
                const int xm = std::max(0, x - 1), xp = std::min(width - 1, x + 1);
                auto at = [&](int yy, int xx) { return static_cast<int>(src[static_cast<size_t>(yy) * width + xx]); };
                const int s = at(ym, xm) + 2 * at(ym, x) + at(ym, xp) + 2 * at(y, xm) + 4 * at(y, x) +
                              2 * at(y, xp) + at(yp, xm) + 2 * at(yp, x) + at(yp, xp);
                image[static_cast<size_t>(y) * width + x] = static_cast<uint8_t>((s + 8) >> 4);
            }
        }
    }
    if (spec.sigma > 0.0) {
        const uint64_t key = splitmix64(seed ^ 0x5bd1e9955bd1e995ull);
        const size_t n = static_cast<size_t>(width) * height;
        for (size_t i = 0; i < n; ++i) {
            const double v = image[i] + spec.sigma * normal_from_hash(splitmix64(key + i));
            const double r = std::floor(v + 0.5);
            image[i] = static_cast<uint8_t>(r < 0.0 ? 0.0 : (r > 255.0 ? 255.0 : r));
        }
    }
    return count;
}

SceneSpec spec_for(int scene_set, int frame_index, Rng& choose) {
    SceneSpec s;
    switch (scene_set) {
        case 1:
            break;
        case 2:
        case 4:
            s.sigma = 6.0;
            s.n36 = 6;
            s.n16 = 2;
            s.side_min = 20.0;
            s.side_max = 200.0;
            s.blur = (frame_index % 2) == 1;
            s.decoys = (frame_index % 4) == 3 ? 2 : 0;
            s.glyphs = (frame_index % 8) == 5 ? 700 : 0;
            break;
        case 3: {
            s.sigma = choose.uniform(2.0, 8.0);
            const int n = choose.range(4, 24);
            s.n16 = choose.range(0, n);
            s.n36 = n - s.n16;
            s.side_min = 16.0;
            s.side_max = 300.0;
            break;
        }
        case 5: {
            s.sigma = choose.uniform(2.0, 8.0);
            s.blank = choose.range(0, 9) == 0;
            const int n = s.blank ? 0 : choose.range(0, 40);
            s.n16 = choose.range(0, n);
            s.n36 = n - s.n16;
            s.side_min = 16.0;
            s.side_max = 300.0;
            break;
        }
        default:
            break;
    }
    return s;
}

}  // namespace

extern "C" {

__attribute__((visibility("default"))) void bds_make_pose(double cx, double cy, double size_px,
                                                          double angle, double perspective,
                                                          double out[9]) {
    const Mat3 m = make_pose(cx, cy, size_px, angle, perspective);
    std::memcpy(out, m.v, sizeof(m.v));
}

// Renders one tag over a white frame exactly as the reference's test
// renderer does; `code` replaces the family codeword when use_code != 0.
__attribute__((visibility("default"))) int bds_render_tag(int family, int id, int width, int height,
                                                          const double pose[9], int supersample,
                                                          uint64_t code, int use_code,
                                                          int flip_one_bit, uint8_t* out) {
    if (family < 0 || family > 1 || !out || width <= 0 || height <= 0) return -1;
    if (!use_code && (id < 0 || id >= kFam[family].count)) return -1;
    Mat3 m;
    std::memcpy(m.v, pose, sizeof(m.v));
    std::memset(out, 255, static_cast<size_t>(width) * height);
    render_patch(family, use_code ? code : kFam[family].codes[id], width, height, m, supersample,
                 flip_one_bit != 0, out);
    return 0;
}

// The reference benchmark scene set: count frames of width x height into
// images (count*W*H bytes), tag ids into ids (count*8) and the -0.5 px
// ground-truth corners into corners (count*8*8 doubles).
__attribute__((visibility("default"))) int bds_ref_scenes(int width, int height, int count,
                                                          uint32_t seed, uint8_t* images,
                                                          int32_t* ids, double* corners) {
    static const int kIds[8] = {0, 3, 7, 11, 17, 42, 101, 586};
    static const double kScale[8] = {1.00, 0.85, 0.70, 1.12, 0.95, 0.60, 1.05, 0.30};
    static const double kPi = 3.14159265358979323846;
    const double base_size = width / 9.0;
    const size_t frame = static_cast<size_t>(width) * height;
    for (int s = 0; s < count; ++s) {
        uint32_t rng = seed + 0x9e3779b9u * static_cast<uint32_t>(s + 1);
        std::vector<uint8_t> image(frame, 255);
        for (int t = 0; t < 8; ++t) {
            const int col = t % 4;
            const int row = t / 4;
            const double cx = (col + 0.5) / 4.0 * width + (next_unit(rng) - 0.5) * 0.05 * width;
            const double cy = (row + 0.5) / 2.0 * height + (next_unit(rng) - 0.5) * 0.06 * height;
            const double size = base_size * kScale[t] * (0.92 + 0.16 * next_unit(rng));
            const double angle = (next_unit(rng) - 0.5) * (0.8 * kPi / 2.0);
            const double perspective = (next_unit(rng) - 0.5) * 1.2e-3;
            const Mat3 pose = make_pose(cx, cy, size, angle, perspective);
            ref_render_into(image, width, height, 0, kCodewords36h11[kIds[t]], pose);
            ids[s * 8 + t] = kIds[t];
            double c[4][2];
            ref_square(pose, c);
            for (int k = 0; k < 4; ++k) {
                corners[(s * 8 + t) * 8 + 2 * k] = c[k][0];
                corners[(s * 8 + t) * 8 + 2 * k + 1] = c[k][1];
            }
        }
        if (s % 8 == 3) {
            const double dx[2] = {width * 0.30, width * 0.70};
            const double dy[2] = {height * 0.50, height * 0.50};
            const double ds[2] = {base_size * 0.50, base_size * 0.40};
            for (int k = 0; k < 2; ++k) {
                const Mat3 pose = make_pose(dx[k], dy[k], ds[k], next_unit(rng) * 0.6, 0.0);
                ref_render_into(image, width, height, 0, ref_non_tag_code(rng, 0, 8), pose);
            }
        }
        uint32_t state = (seed + static_cast<uint32_t>(s)) | 1u;
        for (uint8_t& px : image) {
            state = mix32(state);
            const int delta = static_cast<int>((state >> 28) & 7u) - 3;
            const int value = static_cast<int>(px) + delta;
            px = static_cast<uint8_t>(value < 0 ? 0 : (value > 255 ? 255 : value));
        }
        std::memcpy(images + static_cast<size_t>(s) * frame, image.data(), frame);
    }
    return 0;
}

// One frame of scene set `scene_set` (1, 2, 3, 4 or 5) with the
// given seed.  Returns the number of real tags written to `tags` (each 72
// bytes: family, id, 4 corners as doubles).
__attribute__((visibility("default"))) int bds_render_scene(int scene_set, uint64_t seed,
                                                             int frame_index, int width, int height,
                                                             uint8_t* image, void* tags, int max_tags) {
    if (!image || width < 16 || height < 16) return -1;
    Rng choose{splitmix64(seed * 0x2545f4914f6cdd1dull + 17)};
    const SceneSpec spec = spec_for(scene_set, frame_index, choose);
    return render_scene(spec, seed, width, height, image, static_cast<Tag*>(tags), max_tags);
}

// Renders frames [0, count) of a scene set on `threads` host threads:
// frame i uses seed base_seed + i and size widths[i] x heights[i], packed
// back to back into images.  tag_counts[i] receives the tag count and tags
// gets max_tags records per frame.
__attribute__((visibility("default"))) int bds_render_many(int scene_set, uint64_t base_seed, int count,
                                                           const int32_t* widths,
                                                           const int32_t* heights, uint8_t* images,
                                                           void* tags, int max_tags,
                                                           int32_t* tag_counts, int threads) {
    std::vector<size_t> offsets(static_cast<size_t>(count) + 1, 0);
    for (int i = 0; i < count; ++i) {
        offsets[i + 1] = offsets[i] + static_cast<size_t>(widths[i]) * heights[i];
    }
    std::vector<std::thread> pool;
    const int n = std::max(1, threads);
    for (int t = 0; t < n; ++t) {
        pool.emplace_back([&, t]() {
            for (int i = t; i < count; i += n) {
                tag_counts[i] = bds_render_scene(
                    scene_set, base_seed + static_cast<uint64_t>(i), i, widths[i], heights[i],
                    images + offsets[i], static_cast<Tag*>(tags) + static_cast<size_t>(i) * max_tags,
                    max_tags);
            }
        });
    }
    for (auto& th : pool) th.join();
    return 0;
}

}  // extern "C"
