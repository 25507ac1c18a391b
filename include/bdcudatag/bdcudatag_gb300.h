/*
 * bdcudatag GB300 additions.  These entry points have no counterpart in the
 * reference C ABI; the reference symbols in bdcudatag.h are unchanged.
 *
 * Batches: a bd_batch is a fixed set of cameras (frame size + family set)
 * whose frames are detected together, one launch per pipeline stage for the
 * whole set, replayed as one CUDA graph.  Each camera's results are exactly
 * what a bd_detector of that size and family returns for the same frame.
 */
#ifndef BDCUDATAG_BDCUDATAG_GB300_H
#define BDCUDATAG_BDCUDATAG_GB300_H

#include <stdint.h>

#include "bdcudatag/bdcudatag.h"

#ifdef __cplusplus
extern "C" {
#endif

#define BD_BATCH_MAX_CAMERAS 64
#define BD_FAMILY_MASK(f) (1u << (f))

typedef struct bd_batch bd_batch;

/* One camera of a batch, 16 bytes.  families is a mask of
 * BD_FAMILY_MASK(BD_FAMILY_TAG36H11) and/or BD_FAMILY_MASK(BD_FAMILY_TAG16H5);
 * stages up to candidate selection run once per frame, quad refinement and
 * decoding once per requested family. */
typedef struct bd_camera {
    int32_t width;
    int32_t height;
    uint32_t families;
    int32_t reserved;
} bd_camera;

/* Creates a batch of `count` cameras (1..64).  All device and pinned memory
 * is allocated here.  NULL on failure, with *status_out and bd_last_error()
 * set as for bd_detector_create. */
BD_API bd_batch* bd_batch_create(const bd_camera* cameras, int32_t count, const bd_config* config,
                                 int32_t* status_out);
BD_API void bd_batch_destroy(bd_batch* batch);
BD_API int32_t bd_batch_camera_count(const bd_batch* batch);
BD_API int32_t bd_batch_max_detections(const bd_batch* batch);
/* Device memory held by the batch, in bytes. */
BD_API int64_t bd_batch_device_bytes(const bd_batch* batch);

/*
 * Detects one frame per camera.  frames[i] (row stride strides[i] >= width)
 * is camera i's 8-bit frame: host memory for _host, device memory of the
 * batch's CUDA context for _device.  out receives count * 2 * max_detections
 * records laid out [camera][family][max_detections]; found receives
 * count * 2 entries: the number of detections of camera i, family f at
 * found[2 * i + f] (sorted by id as bd_detector_detect_host), or -1 when the
 * camera does not request that family.  Returns BD_OK or a negative
 * bd_status.
 */
BD_API int32_t bd_batch_detect_host(bd_batch* batch, const uint8_t* const* frames,
                                    const int32_t* strides, bd_detection* out, int32_t* found);
BD_API int32_t bd_batch_detect_device(bd_batch* batch, const uint8_t* const* frames,
                                      const int32_t* strides, bd_detection* out, int32_t* found);

/* Split form of the calls above: submit enqueues the batch and returns at
 * once; wait blocks until it finishes and writes out / found.  One batch may
 * be in flight per bd_batch; use several batches to overlap. */
BD_API int32_t bd_batch_submit_host(bd_batch* batch, const uint8_t* const* frames,
                                    const int32_t* strides);
BD_API int32_t bd_batch_submit_device(bd_batch* batch, const uint8_t* const* frames,
                                      const int32_t* strides);
BD_API int32_t bd_batch_wait(bd_batch* batch, bd_detection* out, int32_t* found);
/* 1 when no batch is in flight or the one in flight has finished (wait then
 * returns at once), 0 while it runs, a negative bd_status on error. */
BD_API int32_t bd_batch_query(bd_batch* batch);

/* Later submits of this batch are enqueued on `cuda_stream` (a
 * cudaStream_t of the batch's device; NULL: the batch's own stream), so a
 * caller can order detection after its own work and time it with its own
 * events.  Several batches on several streams run concurrently. */
BD_API int32_t bd_batch_set_stream(bd_batch* batch, void* cuda_stream);

/* Launch shapes of a batch.  None of them changes any result; they only
 * trade parallelism against per-CTA work:
 *   stats_rows        tile rows per CTA of the tile-statistics kernel: 1, 2, 4
 *   quad_warps        warps per CTA of the fit-and-decode kernel, one
 *                     (candidate, family) per warp: 2, 4, 8
 *   quad_ctas_per_sm  persistent fit-and-decode grid, CTAs per SM (1..32)
 *   quad_split        candidates whose bounding box has a side above this
 *                     many pixels are fitted and decoded by a whole CTA on a
 *                     parallel branch instead (0: none; 0..4096)
 *   band_cap          runs of an 8-row band labelled in shared memory
 *                     (256..2048); a band with more takes the global path
 *   fit_merged        1: big and small candidates are fitted and decoded by
 *                     one launch (no parallel branch in the graph); 0: two
 *                     launches, the big candidates' on a parallel branch
 *   persistent        0: one launch per stage (a CUDA graph of seven or
 *                     eight kernels); 1: the whole batch as one persistent
 *                     kernel whose CTAs pull (frame, stage, unit) items from
 *                     a device work queue.  Same results either way.
 *   persist_ctas      CTAs of the persistent launch (0: every SM's resident
 *                     maximum; 1..65536) */
typedef struct bd_launch_config {
    int32_t stats_rows;
    int32_t quad_warps;
    int32_t quad_ctas_per_sm;
    int32_t quad_split;
    int32_t band_cap;
    int32_t fit_merged;
    int32_t persistent;
    int32_t persist_ctas;
} bd_launch_config;

BD_API int32_t bd_batch_get_launch(const bd_batch* batch, bd_launch_config* out);
/* Sets the launch shapes and re-captures the batch's CUDA graphs. */
BD_API int32_t bd_batch_set_launch(bd_batch* batch, const bd_launch_config* launch);
/* Autotuner: times candidate launch shapes on `iterations` runs of the given
 * device frames (coordinate descent over the five shapes, median GPU time
 * per batch) and keeps the fastest; writes it to best_out and its time to
 * best_ms_out (either may be NULL). */
BD_API int32_t bd_batch_autotune(bd_batch* batch, const uint8_t* const* frames_device,
                                 const int32_t* strides, int32_t iterations,
                                 bd_launch_config* best_out, float* best_ms_out);

/* Test hook of the persistent launch: sets how long a CTA waits for a work
 * queue item before the launch gives up (timeout_ns > 0; default one second)
 * and, with stall_frame >= 0, withholds one work item of that frame, so that
 * a wait runs out: the batch then ends with BD_ERROR_CUDA and
 * "persistent launch gave up: a work-queue wait timed out", and the CUDA
 * context stays usable.  stall_frame -1 restores normal operation. */
BD_API int32_t bd_batch_debug_persist(bd_batch* batch, int64_t timeout_ns, int32_t stall_frame);

/* Pipeline stages, in launch order (for bd_batch_profile_device). */
BD_API int32_t bd_stage_count(void);
BD_API const char* bd_stage_name(int32_t stage);

/* Runs one device-input batch synchronously without the CUDA graph, with
 * CUDA events between kernels, and writes each stage's time in ms to
 * stage_ms[bd_stage_count()].  Results are as for bd_batch_detect_device. */
BD_API int32_t bd_batch_profile_device(bd_batch* batch, const uint8_t* const* frames,
                                       const int32_t* strides, float* stage_ms);

/*
 * Pipelined run of many batches from native code: `steps` batches go round-
 * robin over the `count` bd_batch objects (each keeps its own stream, see
 * bd_batch_set_stream), so up to `count` run on the GPU at once.  Batch k
 * uses frame set k % sets: frames[(k % sets) * cameras + i] is camera i's
 * frame (device pointers when device != 0, else host), strides[i] its stride.
 * All batches must have the same cameras.  Results stay in each batch (read
 * them with bd_batch_wait after the last step if needed).  latency_ms (steps
 * entries, or NULL) receives submit-to-completion time per batch; wall_ms
 * the host time of the whole run.
 */
BD_API int32_t bd_batch_pipeline(bd_batch* const* batches, int32_t count,
                                 const uint8_t* const* frames, const int32_t* strides,
                                 int32_t sets, int32_t steps, int32_t device, float* latency_ms,
                                 double* wall_ms);

/* Pinned host staging buffer of camera i (width * height bytes, stride =
 * width).  A frame written here is submitted without the staging copy by
 * passing this pointer as frames[i]. */
BD_API uint8_t* bd_batch_host_frame(bd_batch* batch, int32_t camera);

/* GPU time of the last completed batch (events around the graph), ms. */
BD_API float bd_batch_last_gpu_ms(const bd_batch* batch);

/* Pipeline counters of camera i in the last batch: [0] candidates before
 * the cap, [1] 0, [2] runs, [3] quads, [4] ROI tile rows. */
BD_API int32_t bd_batch_counts(const bd_batch* batch, int32_t camera, uint32_t counts[5]);

/*
 * Test hook: copies a named intermediate buffer of camera i of the last
 * batch (for a bd_detector: its single frame) into dst.  Returns the
 * buffer's size in bytes, or -1 for an unknown name.  Names: tile_min,
 * tile_max, bits, row_count, runs, label, area, bbox, candidates,
 * hull_quads, quads, decodes, state.
 */
BD_API int64_t bd_batch_debug_stage(bd_batch* batch, int32_t camera, const char* name, void* dst,
                                    int64_t dst_bytes);
BD_API int64_t bd_detector_debug_stage(bd_detector* detector, const char* name, void* dst,
                                       int64_t dst_bytes);

/*
 * Continuous-batching server.  No counterpart in the reference.
 *
 * Frames of several cameras are submitted at any time; a scheduler thread
 * launches a batch whenever one of its preallocated batch plans is free,
 * taking the oldest waiting frame of every camera (cameras with nothing
 * waiting sit that launch out), so frames that arrive while batches run join
 * the next launch and up to `plans` batches overlap on the GPU.  Plans are
 * created at bd_server_create, as many as device_budget_bytes holds (at most
 * max_batches): that is the admission limit.  Each result equals what a
 * bd_detector of the camera's size and family returns for the frame.
 *
 * bd_server_submit returns a ticket (>= 0), or BD_ERROR_OUT_OF_MEMORY when
 * the camera already has queue_depth frames waiting or running.  A frame in
 * page-locked host memory is read in place (keep it unchanged until its
 * ticket completes); other frames are copied at submit.  bd_server_wait /
 * bd_server_poll return 1 with the results (out: 2 * max_detections records,
 * family-major; found[2], -1 for a family the camera does not decode;
 * latency_ms from submit to results), 0 from poll while pending, or a
 * negative bd_status.  A ticket is collected once.
 */
typedef struct bd_server bd_server;

typedef struct bd_server_stats {
    uint64_t submitted;
    uint64_t completed;
    uint64_t rejected;
    uint64_t batches;
    double mean_batch_frames;
    int32_t plans;
    int32_t peak_inflight;
    int64_t device_bytes;
} bd_server_stats;

BD_API bd_server* bd_server_create(const bd_camera* cameras, int32_t count, const bd_config* config,
                                   int64_t device_budget_bytes, int32_t max_batches,
                                   int32_t queue_depth, int32_t* status_out);
BD_API void bd_server_destroy(bd_server* server);
BD_API int64_t bd_server_submit(bd_server* server, int32_t camera, const uint8_t* gray,
                                int32_t stride);
BD_API int32_t bd_server_wait(bd_server* server, int64_t ticket, bd_detection* out, int32_t* found,
                              double* latency_ms);
BD_API int32_t bd_server_poll(bd_server* server, int64_t ticket, bd_detection* out, int32_t* found,
                              double* latency_ms);
BD_API int32_t bd_server_get_stats(bd_server* server, bd_server_stats* out);

/*
 * Photometric corner refinement.  No counterpart in the reference; the
 * reference's edge-line fit stays the default inside detection.
 *
 * For quad q with corners c (TL TR BR BL, pixel-index coordinates, as in
 * bd_detection), H(c) is the square-to-quad homography of the decoder and
 * the template is the tag's cell grid plus a one-cell quiet zone (`cells`
 * per side: 10 for tag36h11, 8 for tag16h5; bd_tag_template builds it),
 * sampled at samples_per_cell^2 points per cell.  Residual of sample s:
 *     r_s = I(H(c) * (u_s, v_s)) - (black + (white - black) * template_s)
 * with I the frame sampled bilinearly; samples that leave the frame are 0.
 * Loss per quad = 0.5 * sum_s r_s^2.  All pointers are device memory;
 * calls are asynchronous on cuda_stream.
 */
typedef struct bd_refine_args {
    const uint8_t* images;       /* frames, image_pitch bytes apart */
    int64_t image_pitch;
    int32_t width;
    int32_t height;
    int32_t stride;              /* row stride in bytes (>= width) */
    int32_t count;               /* number of quads */
    const int32_t* image_index;  /* frame of each quad, or NULL: frame 0 */
    const float* corners;        /* count * 8 */
    const uint8_t* templates;    /* count * cells * cells, 1 = white */
    const float* levels;         /* count * 2 (black, white), or NULL: 0 and 255 */
    int32_t cells;
    int32_t samples_per_cell;
} bd_refine_args;

/* Writes the (bits + 4)^2 cell template of tag `id` (1 = white: quiet zone
 * ring, black border ring, data cells row-major) and returns bits + 4, or a
 * negative bd_status. */
BD_API int32_t bd_tag_template(int32_t family, int32_t id, uint8_t* cells_out);
/* residuals: count * cells^2 * samples_per_cell^2 (or NULL); loss: count. */
BD_API int32_t bd_refine_forward(const bd_refine_args* args, float* residuals, float* loss,
                                 void* cuda_stream);
/* Adjoint: given dL/dr for every residual, writes dL/dcorners (count * 8)
 * and, when grad_images is not NULL, ADDS dL/dI into it (float frames laid
 * out like `images`, pitch image_pitch elements, row stride `stride`). */
BD_API int32_t bd_refine_backward(const bd_refine_args* args, const float* grad_residuals,
                                  float* grad_corners, float* grad_images, void* cuda_stream);
/* Gauss-Newton on the corners, `iterations` damped steps in one launch;
 * with levels NULL the black / white levels are re-estimated from the
 * template cells every step.  loss (count, or NULL) receives the final
 * loss. */
BD_API int32_t bd_refine_gauss_newton(const bd_refine_args* args, float* corners_inout,
                                      int32_t iterations, float* loss, void* cuda_stream);

/*
 * Tile statistics of one frame, for callers that cannot allocate memory.
 * No counterpart in the reference.
 *
 * Who needs it: code that must not call cudaMalloc (or any allocating
 * routine) when it runs -- a camera or ISP callback that may not block, a
 * system that fixes its memory at start-up (real-time, safety-certified), a
 * plugin living inside another framework's allocator.  Detectors and batches
 * allocate at creation; this entry point allocates nothing ever: it uses the
 * caller's buffers plus a 2 KiB scratch array compiled into the library,
 * which every GPU that loads the library holds until the process exits.
 *
 * Computes what the first pipeline stage of a detector computes for the
 * frame gray_device (device memory, rows `stride` bytes apart):
 *   tile_min_device, tile_max_device: ceil(width/8) * ceil(height/8) bytes
 *     each, the minimum / maximum of every 8x8 tile, row-major;
 *   frame_device[0..2]: noise-floor span quartile, Otsu level, ROI tile rows.
 * All buffers are device memory of the current device; the work is enqueued
 * on cuda_stream (NULL: the legacy default stream) and the call returns
 * without waiting.  Frames up to BD_NOALLOC_MAX_WIDTH x BD_NOALLOC_MAX_HEIGHT
 * are accepted; larger ones return BD_ERROR_INVALID_ARGUMENT.
 *
 * Every call looks up the scratch array's device address on the current
 * device (cudaGetSymbolAddress, which allocates nothing), so the address
 * stays right after a device reset.  The first call on a device may load the
 * library's GPU code there; make that first call before capturing a stream.
 * Every call shares the one scratch array per device and clears it first:
 * calls whose GPU work overlaps race and must be serialised by the caller.
 */
#define BD_NOALLOC_MAX_WIDTH 8192
#define BD_NOALLOC_MAX_HEIGHT 16384
BD_API int32_t bd_tile_stats_device_noalloc(const uint8_t* gray_device, int32_t width,
                                            int32_t height, int32_t stride,
                                            uint8_t* tile_min_device, uint8_t* tile_max_device,
                                            uint32_t* frame_device, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(bd_camera) == 16, "bd_camera layout changed");
static_assert(sizeof(bd_server_stats) == 56, "bd_server_stats layout changed");
static_assert(sizeof(bd_refine_args) == 72, "bd_refine_args layout changed");
static_assert(sizeof(bd_launch_config) == 32, "bd_launch_config layout changed");
#endif

#endif /* BDCUDATAG_BDCUDATAG_GB300_H */
