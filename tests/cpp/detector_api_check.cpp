// Drives the C++ API (include/bdcudatag/detector.hpp) the way the reference's
// own C++ callers do (detector/tests/test_detector.cpp, detector/bench/
// bench_detector.cpp): construct, detect from host and device memory, move,
// read the statistics, and provoke the documented exceptions.  Reads one
// frame from a file ("W H" header line, then W*H bytes) and prints one line
// per detection ("det id hamming margin x0 y0 ... x3 y3 h0 ... h8", floats as
// their bit patterns in hex) plus "check <name> ok" lines; tests/
// test_gpu_cpp_api.py compares them with the CPU oracle.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "bdcudatag/detector.hpp"

namespace {

uint32_t bits(float v) {
    uint32_t u;
    std::memcpy(&u, &v, 4);
    return u;
}

void print(const std::vector<bdcudatag::Detection>& dets) {
    for (const auto& d : dets) {
        std::printf("det %d %d %08x", d.id, d.hamming, bits(d.decision_margin));
        for (const auto& c : d.corners) std::printf(" %08x %08x", bits(c[0]), bits(c[1]));
        for (float h : d.homography) std::printf(" %08x", bits(h));
        std::printf("\n");
    }
}

bool same(const std::vector<bdcudatag::Detection>& a, const std::vector<bdcudatag::Detection>& b) {
    if (a.size() != b.size()) return false;
    for (size_t i = 0; i < a.size(); ++i) {
        if (a[i].id != b[i].id || bits(a[i].decision_margin) != bits(b[i].decision_margin)) return false;
        for (int k = 0; k < 4; ++k) {
            if (bits(a[i].corners[k][0]) != bits(b[i].corners[k][0]) ||
                bits(a[i].corners[k][1]) != bits(b[i].corners[k][1]))
                return false;
        }
    }
    return true;
}

int fail(const char* what) {
    std::printf("FAIL %s\n", what);
    return 1;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return fail("usage: detector_api_check <frame file> <family 0|1>");
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return fail("open");
    int w = 0, h = 0;
    if (std::fscanf(f, "%d %d", &w, &h) != 2) return fail("header");
    std::fgetc(f);
    std::vector<uint8_t> img(static_cast<size_t>(w) * h);
    if (std::fread(img.data(), 1, img.size(), f) != img.size()) return fail("pixels");
    std::fclose(f);
    const auto family = std::atoi(argv[2]) == 0 ? bdcudatag::Family::Tag36h11 : bdcudatag::Family::Tag16h5;

    bdcudatag::Detector det(family, w, h);
    const std::vector<bdcudatag::Detection> host = det.detect(img.data(), w);
    print(host);

    // Fixed-capacity overload: the first detection only.
    bdcudatag::Detection one[1];
    const int n1 = det.detect(img.data(), w, one, 1);
    if (n1 != (host.empty() ? 0 : 1) || (n1 == 1 && one[0].id != host[0].id)) return fail("capacity");
    std::printf("check capacity ok\n");

    // Device input, through a row-padded buffer.
    const int pitch = w + 64;
    uint8_t* dev = nullptr;
    if (cudaMalloc(&dev, static_cast<size_t>(pitch) * h) != cudaSuccess) return fail("cudaMalloc");
    cudaMemcpy2D(dev, pitch, img.data(), w, w, h, cudaMemcpyHostToDevice);
    std::vector<bdcudatag::Detection> on_dev(64);
    on_dev.resize(static_cast<size_t>(det.detectDevice(dev, pitch, on_dev.data(), 64)));
    cudaFree(dev);
    if (!same(on_dev, host)) return fail("device");
    std::printf("check device ok\n");

    // Moves keep the detector working; the source throws.
    bdcudatag::Detector moved(std::move(det));
    if (!same(moved.detect(img.data(), w), host)) return fail("move construct");
    bool threw = false;
    try {
        det.detect(img.data(), w);
    } catch (const std::runtime_error& e) {
        threw = std::string(e.what()) == "detector has been moved from";
    }
    if (!threw) return fail("moved-from");
    bdcudatag::Detector other(family, 64, 64);
    other = std::move(moved);
    if (!same(other.detect(img.data(), w), host) || other.width() != w) return fail("move assign");
    std::printf("check move ok\n");

    threw = false;
    try {
        other.detect(img.data(), w, nullptr, 4);
    } catch (const std::invalid_argument&) {
        threw = true;
    }
    if (!threw) return fail("invalid output buffer");
    threw = false;
    try {
        bdcudatag::Detector bad(family, 0, 0);
    } catch (const std::runtime_error&) {
        threw = true;
    }
    if (!threw) return fail("bad dimensions");
    std::printf("check exceptions ok\n");

    const bdcudatag::Stats st = other.stats();
    // host, capacity, device, moved, assigned: five frames on this handle
    if (st.frames != 5 || st.detections != static_cast<int>(host.size())) return fail("stats");
    std::printf("check stats ok\n");
    return 0;
}
