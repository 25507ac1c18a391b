// Host engine: arena allocation, pinned staging, CUDA graphs and result
// copies for a plan of frames (the reference's GpuDetector::Impl,
// gpu_detector.cu:1784-2254, generalised from one frame to a batch).
//
// Memory: one cudaMalloc per plan holds every per-frame buffer, carved at
// 256-byte alignment; the per-frame state records and the result records
// are each contiguous, so a batch costs one memset node and one result copy.
// Detect calls never allocate.

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <sstream>

#include "engine.h"
#include "pipeline.cuh"

namespace bdgb {

namespace {

std::string cuda_error(const char* what, cudaError_t status) {
    std::ostringstream ss;
    ss << what << ": " << cudaGetErrorString(status);
    return ss.str();
}

int next_power_of_two(int v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

PlanConfig resolve_config(const bd_config* config) {
    bd_config c;
    bd_config_init(&c);
    if (config) c = *config;
    PlanConfig p;
    for (int f = 0; f < 2; ++f) {
        p.max_hamming[f] = c.max_hamming >= 0 ? std::min(c.max_hamming, 3) : (f == 0 ? 2 : 1);
    }
    p.min_cluster_pixels = std::max(c.min_cluster_pixels, 1);
    p.min_tag_pixels = std::max(c.min_tag_pixels, 4);
    p.max_detections = std::min(std::max(c.max_detections, 1), kMaxDetectionsCap);
    p.max_candidates = c.max_candidates;
    p.refine_edges = c.refine_edges != 0;
    p.use_graph = c.use_cuda_graph != 0;
    p.min_decision_margin = c.min_decision_margin;
    p.decode_sharpening = c.decode_sharpening;
    return p;
}

int auto_max_candidates(int width, int height, int configured) {
    if (configured > 0) return std::min(std::max(configured, 16), 1024);
    return std::min(std::max(next_power_of_two((width * height) / 4096) * 3 / 2, 96), 1024);
}

struct Plan::Impl {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t branch = nullptr;      // parallel branch: big-candidate kernel
    cudaEvent_t ev_fork = nullptr;
    cudaEvent_t ev_join = nullptr;
    cudaEvent_t ev_start = nullptr;
    cudaEvent_t ev_stop = nullptr;
    void* arena = nullptr;
    BatchDesc host_desc{};
    BatchDesc* dev_desc = nullptr;
    FrameIO* io_fixed = nullptr;     // device: arena frame buffers
    FrameIO* io_caller = nullptr;    // device: caller pointers, device path
    FrameIO* io_staging = nullptr;   // pinned
    uint8_t* frames_dev = nullptr;
    uint8_t* frames_pinned = nullptr;
    size_t frame_bytes = 0;
    std::vector<size_t> frame_offset;
    FrameState* states = nullptr;
    size_t states_bytes = 0;
    WorkQueue* queue = nullptr;        // right after the states: one memset clears both
    size_t queue_bytes = 0;
    PersistParams persist;
    uint8_t* results_dev = nullptr;
    uint8_t* results_pinned = nullptr;
    size_t results_bytes = 0;
    size_t result_stride = 0;
    cudaGraphExec_t graph_host = nullptr;    // H2D of the staging buffer + pipeline + D2H
    cudaGraphExec_t graph_fixed = nullptr;   // pipeline + D2H on the plan's device frames
    cudaGraphExec_t graph_device = nullptr;  // caller device frames
    cudaStream_t user_stream = nullptr;      // caller stream for submits (null: own stream)
    LaunchConfig launch_cfg;
    int sm_count = 152;
    cudaEvent_t stage_events[kStageCount + 1] = {};
    bool pending = false;

    cudaStream_t active() const { return user_stream ? user_stream : stream; }

    ~Impl() {
        if (stream) cudaStreamSynchronize(stream);
        if (user_stream) cudaStreamSynchronize(user_stream);
        destroy_graphs();
        for (cudaEvent_t e : stage_events) {
            if (e) cudaEventDestroy(e);
        }
        if (branch) cudaStreamSynchronize(branch);
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (branch) cudaStreamDestroy(branch);
        if (ev_start) cudaEventDestroy(ev_start);
        if (ev_stop) cudaEventDestroy(ev_stop);
        if (stream) cudaStreamDestroy(stream);
        if (arena) cudaFree(arena);
        if (frames_pinned) cudaFreeHost(frames_pinned);
        if (results_pinned) cudaFreeHost(results_pinned);
        if (io_staging) cudaFreeHost(io_staging);
    }

    // mode 0: staging H2D + pipeline on the plan's frames; 1: pipeline on
    // the plan's frames (inputs already copied); 2: caller device frames.
    void enqueue(int mode, cudaStream_t s, void* const* events = nullptr) {
        if (mode == 0) {
            cudaMemcpyAsync(frames_dev, frames_pinned, frame_bytes, cudaMemcpyHostToDevice, s);
        } else if (mode == 2) {
            cudaMemcpyAsync(io_caller, io_staging, sizeof(FrameIO) * host_desc.frames,
                            cudaMemcpyHostToDevice, s);
        }
        const FrameIO* io = mode == 2 ? io_caller : io_fixed;
        if (launch_cfg.persistent && !events) {
            cudaMemsetAsync(states, 0, states_bytes + queue_bytes, s);
            enqueue_persistent(dev_desc, host_desc, io, queue, s, launch_cfg, sm_count, persist);
        } else {
            // Stage events (profile_device) always time the per-stage launches.
            cudaMemsetAsync(states, 0, states_bytes, s);
            const ForkJoin fork{branch, ev_fork, ev_join};
            enqueue_pipeline(dev_desc, host_desc, io, s, launch_cfg, sm_count, branch ? &fork : nullptr,
                             events);
        }
        cudaMemcpyAsync(results_pinned, results_dev, results_bytes, cudaMemcpyDeviceToHost, s);
    }

    void launch(int mode, cudaStream_t s) {
        cudaGraphExec_t g = mode == 0 ? graph_host : (mode == 1 ? graph_fixed : graph_device);
        if (g) {
            cudaGraphLaunch(g, s);
        } else {
            enqueue(mode, s);
        }
    }

    void destroy_graphs() {
        if (graph_host) cudaGraphExecDestroy(graph_host);
        if (graph_fixed) cudaGraphExecDestroy(graph_fixed);
        if (graph_device) cudaGraphExecDestroy(graph_device);
        graph_host = graph_fixed = graph_device = nullptr;
    }

    void capture_all() {
        destroy_graphs();
        if (!capture(0, &graph_host)) graph_host = nullptr;
        if (!capture(1, &graph_fixed)) graph_fixed = nullptr;
        if (!capture(2, &graph_device)) graph_device = nullptr;
    }

    bool capture(int mode, cudaGraphExec_t* out) {
        if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        enqueue(mode, stream);
        cudaGraph_t graph = nullptr;
        if (cudaStreamEndCapture(stream, &graph) != cudaSuccess || !graph) {
            cudaGetLastError();
            return false;
        }
        cudaGraphExec_t exec = nullptr;
        const cudaError_t st = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (st != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        *out = exec;
        return true;
    }
};

Plan* Plan::create(const std::vector<PlanFrame>& frames, const PlanConfig& config,
                   std::string* error) {
    if (frames.empty() || frames.size() > static_cast<size_t>(kMaxFrames)) {
        if (error) *error = "a plan holds 1 to 64 frames";
        return nullptr;
    }
    for (const PlanFrame& f : frames) {
        if (f.width < 16 || f.width > BD_MAX_WIDTH || f.height < 16 || f.height > BD_MAX_HEIGHT) {
            if (error) *error = "image dimensions out of range (16..8192 x 16..16384)";
            return nullptr;
        }
        if ((f.families & 3u) == 0 || (f.families & ~3u) != 0) {
            if (error) *error = "family mask must select tag36h11 and/or tag16h5";
            return nullptr;
        }
    }
    Plan* plan = new Plan();
    plan->frames_ = frames;
    plan->config_ = config;
    plan->impl_ = new Impl();
    Impl& im = *plan->impl_;
    auto fail = [&](const std::string& msg) -> Plan* {
        if (error) *error = msg;
        delete plan;
        return nullptr;
    };
    cudaError_t st = cudaGetDevice(&im.device);
    if (st != cudaSuccess) return fail(cuda_error("cudaGetDevice", st));
    if (prepare_pipeline() != 0 || prepare_persistent() != 0) {
        cudaGetLastError();
        return fail("cudaFuncSetAttribute failed");
    }
    cudaDeviceGetAttribute(&im.sm_count, cudaDevAttrMultiProcessorCount, im.device);

    const int nf = static_cast<int>(frames.size());
    const int md = config.max_detections;
    // --- sizes and arena layout ---
    struct Carve {
        size_t off = 0;
        size_t take(size_t bytes) {
            const size_t at = off;
            off = align_up(off + std::max<size_t>(bytes, 1), 256);
            return at;
        }
    } carve;
    BatchDesc& hd = im.host_desc;
    std::memset(&hd, 0, sizeof(hd));
    hd.frames = nf;
    std::vector<size_t> off_frame(nf), off_tmin(nf), off_tmax(nf), off_lo(nf), off_hi(nf),
        off_bits(nf), off_rc(nf), off_runs(nf), off_parent(nf), off_area(nf), off_bbox(nf),
        off_meta(nf), off_bands(nf), off_cands(nf), off_hull(nf), off_quads(nf), off_dec(nf),
        off_lroots(nf), off_lcount(nf), off_mode(nf), off_fit(nf);
    im.frame_offset.resize(nf);
    size_t frame_total = 0;
    for (int i = 0; i < nf; ++i) {
        im.frame_offset[i] = frame_total;
        frame_total += align_up(static_cast<size_t>(frames[i].width) * frames[i].height, 256);
    }
    im.frame_bytes = frame_total;
    const size_t frames_at = carve.take(frame_total);
    im.states_bytes = sizeof(FrameState) * nf;
    uint32_t queue_capacity = 0;
    for (const PlanFrame& f : frames) {
        queue_capacity += queue_items_per_frame((f.height + kTile - 1) / kTile,
                                                auto_max_candidates(f.width, f.height, config.max_candidates));
    }
    im.queue_bytes = offsetof(WorkQueue, items) + sizeof(uint32_t) * queue_capacity;
    static_assert(sizeof(FrameState) % 16 == 0, "the work queue follows the states");
    hd.queue_capacity = queue_capacity;
    const size_t states_at = carve.take(im.states_bytes + im.queue_bytes);
    im.result_stride = align_up(result_bytes(md), 256);
    im.results_bytes = im.result_stride * nf;
    const size_t results_at = carve.take(im.results_bytes);
    const size_t desc_at = carve.take(sizeof(BatchDesc));
    const size_t io_fixed_at = carve.take(sizeof(FrameIO) * nf);
    const size_t io_caller_at = carve.take(sizeof(FrameIO) * nf);
    int bands = 0;
    for (int i = 0; i < nf; ++i) {
        FrameDesc& d = hd.f[i];
        const PlanFrame& f = frames[i];
        d.width = f.width;
        d.height = f.height;
        d.tile_w = (f.width + kTile - 1) / kTile;
        d.tile_h = (f.height + kTile - 1) / kTile;
        d.words = (f.width + 31) / 32;
        d.row_cap = f.width / 2 + 2;
        d.max_candidates = auto_max_candidates(f.width, f.height, config.max_candidates);
        d.max_detections = md;
        d.families = f.families;
        d.min_cluster_pixels = config.min_cluster_pixels;
        d.min_tag_pixels = config.min_tag_pixels;
        d.refine_edges = config.refine_edges ? 1 : 0;
        d.max_hamming[0] = config.max_hamming[0];
        d.max_hamming[1] = config.max_hamming[1];
        d.min_margin = config.min_decision_margin;
        d.sharpening = config.decode_sharpening;
        const size_t T = static_cast<size_t>(d.tile_w) * d.tile_h;
        const size_t slots = static_cast<size_t>(f.height) * d.row_cap;
        const size_t mc = static_cast<size_t>(d.max_candidates);
        hd.band_prefix[i] = bands;
        bands += d.tile_h;
        off_tmin[i] = carve.take(T);
        off_tmax[i] = carve.take(T);
        off_lo[i] = carve.take(sizeof(int32_t) * d.tile_h);
        off_hi[i] = carve.take(sizeof(int32_t) * d.tile_h);
        off_bits[i] = carve.take(sizeof(uint32_t) * d.words * f.height);
        off_rc[i] = carve.take(sizeof(uint32_t) * f.height);
        off_runs[i] = carve.take(sizeof(uint32_t) * slots);
        off_parent[i] = carve.take(sizeof(uint32_t) * slots);
        off_area[i] = carve.take(sizeof(uint32_t) * slots);
        off_bbox[i] = carve.take(sizeof(uint32_t) * 4 * slots);
        off_meta[i] = carve.take(sizeof(uint32_t) * slots);
        off_lroots[i] = carve.take(sizeof(uint32_t) * slots);
        off_lcount[i] = carve.take(sizeof(uint32_t) * d.tile_h);
        off_mode[i] = carve.take(sizeof(uint32_t) * d.tile_h);
        off_bands[i] = carve.take(sizeof(uint32_t) * 64 * d.tile_h);
        off_cands[i] = carve.take(sizeof(uint32_t) * mc);
        off_fit[i] = carve.take(sizeof(uint32_t) * mc);
        off_hull[i] = carve.take(sizeof(float) * 8 * mc);
        off_quads[i] = carve.take(sizeof(float) * 16 * mc);
        off_dec[i] = carve.take(sizeof(DecodeOut) * 2 * mc);
    }
    hd.band_prefix[nf] = bands;
    hd.total_bands = bands;
    set_stats_rows(hd, im.launch_cfg.stats_rows);
    plan->arena_bytes_ = carve.off;

    st = cudaMalloc(&im.arena, carve.off);
    if (st != cudaSuccess) {
        cudaGetLastError();
        return fail(cuda_error("cudaMalloc", st));
    }
    uint8_t* base = static_cast<uint8_t*>(im.arena);
    im.frames_dev = base + frames_at;
    im.states = reinterpret_cast<FrameState*>(base + states_at);
    im.queue = reinterpret_cast<WorkQueue*>(base + states_at + im.states_bytes);
    im.results_dev = base + results_at;
    im.dev_desc = reinterpret_cast<BatchDesc*>(base + desc_at);
    im.io_fixed = reinterpret_cast<FrameIO*>(base + io_fixed_at);
    im.io_caller = reinterpret_cast<FrameIO*>(base + io_caller_at);
    std::vector<FrameIO> fixed(nf);
    for (int i = 0; i < nf; ++i) {
        FrameDesc& d = hd.f[i];
        d.tile_min = base + off_tmin[i];
        d.tile_max = base + off_tmax[i];
        d.row_lo = reinterpret_cast<int32_t*>(base + off_lo[i]);
        d.row_hi = reinterpret_cast<int32_t*>(base + off_hi[i]);
        d.bits = reinterpret_cast<uint32_t*>(base + off_bits[i]);
        d.row_count = reinterpret_cast<uint32_t*>(base + off_rc[i]);
        d.runs = reinterpret_cast<uint32_t*>(base + off_runs[i]);
        d.parent = reinterpret_cast<uint32_t*>(base + off_parent[i]);
        d.area = reinterpret_cast<uint32_t*>(base + off_area[i]);
        d.bbox = reinterpret_cast<uint32_t*>(base + off_bbox[i]);
        d.cand_meta = reinterpret_cast<uint32_t*>(base + off_meta[i]);
        d.lroots = reinterpret_cast<uint32_t*>(base + off_lroots[i]);
        d.lroot_count = reinterpret_cast<uint32_t*>(base + off_lcount[i]);
        d.band_mode = reinterpret_cast<uint32_t*>(base + off_mode[i]);
        d.band_bins = reinterpret_cast<uint32_t*>(base + off_bands[i]);
        d.candidates = reinterpret_cast<uint32_t*>(base + off_cands[i]);
        d.fit_list = reinterpret_cast<uint32_t*>(base + off_fit[i]);
        d.state = im.states + i;
        d.hull_quads = reinterpret_cast<float*>(base + off_hull[i]);
        d.quads = reinterpret_cast<float*>(base + off_quads[i]);
        d.decodes = reinterpret_cast<DecodeOut*>(base + off_dec[i]);
        d.result = reinterpret_cast<FrameResultHeader*>(im.results_dev + im.result_stride * i);
        fixed[i].gray = im.frames_dev + im.frame_offset[i];
        fixed[i].stride = frames[i].width;
    }
    st = cudaHostAlloc(reinterpret_cast<void**>(&im.frames_pinned), frame_total, cudaHostAllocPortable);
    if (st == cudaSuccess)
        st = cudaHostAlloc(reinterpret_cast<void**>(&im.results_pinned), im.results_bytes,
                           cudaHostAllocPortable);
    if (st == cudaSuccess)
        st = cudaHostAlloc(reinterpret_cast<void**>(&im.io_staging), sizeof(FrameIO) * nf,
                           cudaHostAllocPortable);
    if (st != cudaSuccess) {
        cudaGetLastError();
        return fail(cuda_error("cudaHostAlloc", st));
    }
    std::memset(im.results_pinned, 0, im.results_bytes);
    st = cudaStreamCreateWithFlags(&im.stream, cudaStreamNonBlocking);
    if (st == cudaSuccess) st = cudaStreamCreateWithFlags(&im.branch, cudaStreamNonBlocking);
    if (st == cudaSuccess) st = cudaEventCreateWithFlags(&im.ev_fork, cudaEventDisableTiming);
    if (st == cudaSuccess) st = cudaEventCreateWithFlags(&im.ev_join, cudaEventDisableTiming);
    if (st == cudaSuccess) st = cudaEventCreate(&im.ev_start);
    if (st == cudaSuccess) st = cudaEventCreate(&im.ev_stop);
    if (st != cudaSuccess) return fail(cuda_error("cudaStreamCreate", st));
    st = cudaMemcpy(im.dev_desc, &hd, sizeof(BatchDesc), cudaMemcpyHostToDevice);
    if (st == cudaSuccess)
        st = cudaMemcpy(im.io_fixed, fixed.data(), sizeof(FrameIO) * nf, cudaMemcpyHostToDevice);
    if (st == cudaSuccess) st = cudaMemset(im.frames_dev, 0, frame_total);
    if (st == cudaSuccess) st = cudaMemset(im.results_dev, 0, im.results_bytes);
    if (st != cudaSuccess) return fail(cuda_error("cudaMemcpy(plan)", st));
    for (int i = 0; i < nf; ++i) {
        im.io_staging[i].gray = fixed[i].gray;
        im.io_staging[i].stride = fixed[i].stride;
    }
    if (config.use_graph) {
        // A failed capture falls back to direct launches (reference
        // gpu_detector.cu:2051-2056).
        im.capture_all();
    }
    return plan;
}

Plan::~Plan() { delete impl_; }

int Plan::max_candidates(int frame) const { return impl_->host_desc.f[frame].max_candidates; }

uint8_t* Plan::host_frame(int i) { return impl_->frames_pinned + impl_->frame_offset[i]; }

int Plan::submit_host(const uint8_t* const* frames, const int32_t* strides, std::string* error) {
    Impl& im = *impl_;
    if (im.pending) {
        if (error) *error = "a batch is already in flight";
        return -1;
    }
    const cudaStream_t s = im.active();
    // Frames in page-locked memory are copied by DMA straight from the
    // caller; others are compacted into the pinned staging buffer first (the
    // reference's detect_host path, gpu_detector.cu:2169-2176).
    bool direct[kMaxFrames] = {};
    bool any_direct = false;
    for (int i = 0; i < this->frames(); ++i) {
        const int w = frames_[i].width, h = frames_[i].height;
        uint8_t* dst = im.frames_pinned + im.frame_offset[i];
        if (!frames[i]) {
            if (error) *error = "null image pointer";
            return -1;
        }
        if (frames[i] == dst) continue;  // already in the staging buffer
        cudaPointerAttributes attr;
        if (cudaPointerGetAttributes(&attr, frames[i]) == cudaSuccess &&
            attr.type == cudaMemoryTypeHost) {
            direct[i] = any_direct = true;
            continue;
        }
        cudaGetLastError();
        if (strides[i] == w) {
            std::memcpy(dst, frames[i], static_cast<size_t>(w) * h);
        } else {
            for (int y = 0; y < h; ++y) {
                std::memcpy(dst + static_cast<size_t>(y) * w,
                            frames[i] + static_cast<size_t>(y) * strides[i], w);
            }
        }
    }
    cudaEventRecord(im.ev_start, s);
    if (!any_direct) {
        im.launch(0, s);
    } else {
        for (int i = 0; i < this->frames();) {
            const int w = frames_[i].width, h = frames_[i].height;
            uint8_t* dev = im.frames_dev + im.frame_offset[i];
            if (direct[i] && strides[i] == w) {
                // Tightly strided frames that follow one another both in the
                // caller's memory and in the plan's buffer go in one copy.
                size_t bytes = static_cast<size_t>(w) * h;
                int j = i + 1;
                while (j < this->frames() && direct[j] && strides[j] == frames_[j].width &&
                       frames[j] == frames[i] + bytes &&
                       im.frame_offset[j] == im.frame_offset[i] + bytes) {
                    bytes += static_cast<size_t>(frames_[j].width) * frames_[j].height;
                    ++j;
                }
                cudaMemcpyAsync(dev, frames[i], bytes, cudaMemcpyHostToDevice, s);
                i = j;
                continue;
            }
            if (direct[i]) {
                cudaMemcpy2DAsync(dev, w, frames[i], strides[i], w, h, cudaMemcpyHostToDevice, s);
            } else {
                cudaMemcpyAsync(dev, im.frames_pinned + im.frame_offset[i], static_cast<size_t>(w) * h,
                                cudaMemcpyHostToDevice, s);
            }
            ++i;
        }
        im.launch(1, s);
    }
    cudaEventRecord(im.ev_stop, s);
    const cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaGraphLaunch", st);
        return -1;
    }
    im.pending = true;
    return 0;
}

int Plan::submit_device(const uint8_t* const* frames, const int32_t* strides, std::string* error) {
    Impl& im = *impl_;
    if (im.pending) {
        if (error) *error = "a batch is already in flight";
        return -1;
    }
    for (int i = 0; i < this->frames(); ++i) {
        if (!frames[i]) {
            if (error) *error = "null device image pointer";
            return -1;
        }
        im.io_staging[i].gray = frames[i];
        im.io_staging[i].stride = strides[i];
    }
    const cudaStream_t s = im.active();
    cudaEventRecord(im.ev_start, s);
    im.launch(2, s);
    cudaEventRecord(im.ev_stop, s);
    const cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaGraphLaunch", st);
        return -1;
    }
    im.pending = true;
    return 0;
}

int Plan::submit_slots(const uint8_t* const* frames, const int32_t* strides, std::string* error) {
    Impl& im = *impl_;
    if (im.pending) {
        if (error) *error = "a batch is already in flight";
        return -1;
    }
    const cudaStream_t s = im.active();
    cudaEventRecord(im.ev_start, s);
    for (int i = 0; i < this->frames(); ++i) {
        const int w = frames_[i].width, h = frames_[i].height;
        uint8_t* dev = im.frames_dev + im.frame_offset[i];
        if (!frames[i]) {
            im.io_staging[i].gray = nullptr;
            im.io_staging[i].stride = 0;
            continue;
        }
        cudaPointerAttributes attr;
        const bool pinned = cudaPointerGetAttributes(&attr, frames[i]) == cudaSuccess &&
                            attr.type == cudaMemoryTypeHost;
        cudaGetLastError();
        if (pinned) {
            cudaMemcpy2DAsync(dev, w, frames[i], strides[i], w, h, cudaMemcpyHostToDevice, s);
        } else {
            uint8_t* stage = im.frames_pinned + im.frame_offset[i];
            for (int y = 0; y < h; ++y) {
                std::memcpy(stage + static_cast<size_t>(y) * w,
                            frames[i] + static_cast<size_t>(y) * strides[i], w);
            }
            cudaMemcpyAsync(dev, stage, static_cast<size_t>(w) * h, cudaMemcpyHostToDevice, s);
        }
        im.io_staging[i].gray = dev;
        im.io_staging[i].stride = w;
    }
    im.launch(2, s);
    cudaEventRecord(im.ev_stop, s);
    const cudaError_t st = cudaGetLastError();
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaGraphLaunch", st);
        return -1;
    }
    im.pending = true;
    return 0;
}

const LaunchConfig& Plan::launch() const { return impl_->launch_cfg; }

int Plan::set_launch(const LaunchConfig& lc, std::string* error) {
    Impl& im = *impl_;
    if (!(lc.stats_rows == 1 || lc.stats_rows == 2 || lc.stats_rows == 4) ||
        !(lc.quad_warps == 2 || lc.quad_warps == 4 || lc.quad_warps == kMaxQuadWarps) ||
        lc.quad_ctas_per_sm < 1 || lc.quad_ctas_per_sm > 32 || lc.quad_split < 0 ||
        lc.quad_split > 4096 || lc.band_cap < 256 || lc.band_cap > 2048 ||
        !(lc.fit_merged == 0 || lc.fit_merged == 1) || !(lc.persistent == 0 || lc.persistent == 1) ||
        lc.persist_ctas < 0 || lc.persist_ctas > 65536) {
        if (error) *error = "launch config out of range";
        return -1;
    }
    if (im.pending && wait(error) != 0) return -1;
    cudaStreamSynchronize(im.stream);
    im.launch_cfg = lc;
    set_stats_rows(im.host_desc, lc.stats_rows);
    const cudaError_t st = cudaMemcpy(im.dev_desc, &im.host_desc, sizeof(BatchDesc),
                                      cudaMemcpyHostToDevice);
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaMemcpy(plan)", st);
        return -1;
    }
    if (config_.use_graph) im.capture_all();
    return 0;
}

int Plan::autotune(const uint8_t* const* frames, const int32_t* strides, int iterations,
                   float* best_ms, std::string* error) {
    Impl& im = *impl_;
    iterations = std::max(iterations, 3);
    std::vector<float> times(iterations);
    auto measure = [&](const LaunchConfig& lc, float* ms) -> int {
        if (set_launch(lc, error) != 0) return -1;
        for (int k = 0; k < 3; ++k) {
            if (run_device(frames, strides, error) != 0) return -1;
        }
        for (int k = 0; k < iterations; ++k) {
            if (run_device(frames, strides, error) != 0) return -1;
            times[k] = last_gpu_ms_;
        }
        std::vector<float> sorted = times;
        std::sort(sorted.begin(), sorted.end());
        *ms = sorted[sorted.size() / 2];
        return 0;
    };
    LaunchConfig best = im.launch_cfg;
    float best_t = 0.0f;
    if (measure(best, &best_t) != 0) return -1;
    const int stats_rows[] = {1, 2, 4};
    const int quad_warps[] = {2, 4, 8};
    const int quad_ctas[] = {2, 4, 8, 16};
    const int quad_split[] = {32, 48, 64, 96, 0};
    const int band_cap[] = {2048, 1024, 512};
    auto try_values = [&](auto field, const int* values, int n) -> int {
        for (int i = 0; i < n; ++i) {
            LaunchConfig lc = best;
            lc.*field = values[i];
            if (lc.*field == best.*field) continue;
            float t = 0.0f;
            if (measure(lc, &t) != 0) return -1;
            if (t < best_t) {
                best_t = t;
                best = lc;
            }
        }
        return 0;
    };
    if (try_values(&LaunchConfig::stats_rows, stats_rows, 3) != 0) return -1;
    if (try_values(&LaunchConfig::quad_warps, quad_warps, 3) != 0) return -1;
    if (try_values(&LaunchConfig::quad_ctas_per_sm, quad_ctas, 4) != 0) return -1;
    if (try_values(&LaunchConfig::quad_split, quad_split, 5) != 0) return -1;
    if (try_values(&LaunchConfig::band_cap, band_cap, 3) != 0) return -1;
    const int fit_merged[] = {0, 1};
    if (try_values(&LaunchConfig::fit_merged, fit_merged, 2) != 0) return -1;
    const int persistent[] = {0, 1};
    if (try_values(&LaunchConfig::persistent, persistent, 2) != 0) return -1;
    if (set_launch(best, error) != 0) return -1;
    if (best_ms) *best_ms = best_t;
    return 0;
}

int Plan::set_persist_params(int64_t timeout_ns, int stall_frame, std::string* error) {
    Impl& im = *impl_;
    if (timeout_ns <= 0 || stall_frame < -1 || stall_frame >= frames()) {
        if (error) *error = "persistent test parameters out of range";
        return -1;
    }
    if (im.pending && wait(error) != 0) return -1;
    cudaStreamSynchronize(im.stream);
    im.persist.timeout_ns = static_cast<uint64_t>(timeout_ns);
    im.persist.stall_frame = stall_frame;
    if (config_.use_graph) im.capture_all();
    return 0;
}

void Plan::set_stream(void* stream) {
    impl_->user_stream = static_cast<cudaStream_t>(stream);
}

int Plan::profile_device(const uint8_t* const* frames, const int32_t* strides, float* stage_ms,
                         std::string* error) {
    Impl& im = *impl_;
    if (im.pending && wait(error) != 0) return -1;
    for (int k = 0; k <= kStageCount; ++k) {
        if (!im.stage_events[k] && cudaEventCreate(&im.stage_events[k]) != cudaSuccess) {
            if (error) *error = "cudaEventCreate failed";
            return -1;
        }
    }
    for (int i = 0; i < this->frames(); ++i) {
        im.io_staging[i].gray = frames[i];
        im.io_staging[i].stride = strides[i];
    }
    const cudaStream_t s = im.active();
    im.enqueue(2, s, reinterpret_cast<void* const*>(im.stage_events));
    const cudaError_t st = cudaStreamSynchronize(s);
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaStreamSynchronize", st);
        return -1;
    }
    for (int k = 0; k < kStageCount; ++k) {
        cudaEventElapsedTime(&stage_ms[k], im.stage_events[k], im.stage_events[k + 1]);
    }
    return 0;
}

int Plan::wait(std::string* error) {
    Impl& im = *impl_;
    if (!im.pending) return 0;
    im.pending = false;
    const cudaError_t st = cudaEventSynchronize(im.ev_stop);
    if (st != cudaSuccess) {
        if (error) *error = cuda_error("cudaEventSynchronize", st);
        return -1;
    }
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, im.ev_start, im.ev_stop);
    last_gpu_ms_ = ms;
    const cudaError_t late = cudaGetLastError();
    if (late != cudaSuccess) {
        if (error) *error = cuda_error("CUDA launch", late);
        return -1;
    }
    // The persistent launch reports a wait that ran out (or a queue
    // overflow) in every frame's result header.
    for (int i = 0; i < frames(); ++i) {
        const uint32_t status = result(i)->pad;
        if (status) {
            if (error) {
                *error = (status & kQueueTimeout) ? "persistent launch gave up: a work-queue wait timed out"
                                                  : "persistent launch gave up: work queue overflow";
            }
            return -1;
        }
    }
    return 0;
}

int Plan::query(std::string* error) {
    Impl& im = *impl_;
    if (!im.pending) return 1;
    const cudaError_t st = cudaEventQuery(im.ev_stop);
    if (st == cudaSuccess) return 1;
    if (st == cudaErrorNotReady) return 0;
    if (error) *error = cuda_error("cudaEventQuery", st);
    return -1;
}

int Plan::run_host(const uint8_t* const* frames, const int32_t* strides, std::string* error) {
    if (submit_host(frames, strides, error) != 0) return -1;
    return wait(error);
}

int Plan::run_device(const uint8_t* const* frames, const int32_t* strides, std::string* error) {
    if (submit_device(frames, strides, error) != 0) return -1;
    return wait(error);
}

const FrameResultHeader* Plan::result(int frame) const {
    return reinterpret_cast<const FrameResultHeader*>(impl_->results_pinned +
                                                      impl_->result_stride * frame);
}

const bd_detection* Plan::detections(int frame, int family) const {
    return result_detections(const_cast<FrameResultHeader*>(result(frame))) +
           static_cast<size_t>(family) * config_.max_detections;
}

int Plan::found(int frame, int family) const {
    return static_cast<int>(result(frame)->found[family]);
}

int64_t Plan::copy_stage(int frame, const char* name, void* dst, int64_t dst_bytes) {
    Impl& im = *impl_;
    if (frame < 0 || frame >= frames() || !name) return -1;
    const FrameDesc& d = im.host_desc.f[frame];
    const size_t T = static_cast<size_t>(d.tile_w) * d.tile_h;
    const size_t slots = static_cast<size_t>(d.height) * d.row_cap;
    const size_t mc = static_cast<size_t>(d.max_candidates);
    const std::string n(name);
    const void* src = nullptr;
    size_t bytes = 0;
    if (n == "tile_min") { src = d.tile_min; bytes = T; }
    else if (n == "tile_max") { src = d.tile_max; bytes = T; }
    else if (n == "bits") { src = d.bits; bytes = sizeof(uint32_t) * d.words * d.height; }
    else if (n == "row_count") { src = d.row_count; bytes = sizeof(uint32_t) * d.height; }
    else if (n == "runs") { src = d.runs; bytes = sizeof(uint32_t) * slots; }
    else if (n == "label") { src = d.parent; bytes = sizeof(uint32_t) * slots; }
    else if (n == "area") { src = d.area; bytes = sizeof(uint32_t) * slots; }
    else if (n == "bbox") { src = d.bbox; bytes = sizeof(uint32_t) * 4 * slots; }
    else if (n == "candidates") { src = d.candidates; bytes = sizeof(uint32_t) * mc; }
    else if (n == "hull_quads") { src = d.hull_quads; bytes = sizeof(float) * 8 * mc; }
    else if (n == "quads") { src = d.quads; bytes = sizeof(float) * 16 * mc; }
    else if (n == "decodes") { src = d.decodes; bytes = sizeof(DecodeOut) * 2 * mc; }
    else if (n == "state") { src = d.state; bytes = sizeof(FrameState); }
    else return -1;
    if (dst && dst_bytes > 0) {
        cudaStreamSynchronize(im.stream);
        const size_t n_copy = std::min(bytes, static_cast<size_t>(dst_bytes));
        if (cudaMemcpy(dst, src, n_copy, cudaMemcpyDeviceToHost) != cudaSuccess) return -1;
    }
    return static_cast<int64_t>(bytes);
}

}  // namespace bdgb
