/*
 * bdcudatag C ABI, GB300 (sm_103a) implementation.
 *
 * This header is the drop-in boundary: every type, constant and function
 * below has the same name, layout, value and meaning as the reference
 * interface it replaces (reference detector/include/bdcudatag/bdcudatag.h),
 * so the Java FFM binding (java-api .../internal/NativeLibrary.java:104-126)
 * and the Python ctypes mirror (detector/bench/compare_detectors.py:76-156)
 * bind this library unchanged.  New entry points live in bdcudatag_gb300.h.
 *
 * One detector handles one tag family at one fixed image size.
 */
#ifndef BDCUDATAG_BDCUDATAG_H
#define BDCUDATAG_BDCUDATAG_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#if defined(BDCUDATAG_BUILDING)
#define BD_API __declspec(dllexport)
#elif defined(BDCUDATAG_STATIC)
#define BD_API
#else
#define BD_API __declspec(dllimport)
#endif
#else
#define BD_API __attribute__((visibility("default")))
#endif

/* ABI revision and image size limits (reference bdcudatag.h:28-30). */
#define BD_API_VERSION 2u
#define BD_MAX_WIDTH 8192
#define BD_MAX_HEIGHT 16384

typedef struct bd_detector bd_detector;

/* Tag families (reference bdcudatag.h:34-37). */
typedef enum bd_family {
    BD_FAMILY_TAG36H11 = 0,
    BD_FAMILY_TAG16H5 = 1
} bd_family;

/* Status codes returned by the API (reference bdcudatag.h:39-46). */
typedef enum bd_status {
    BD_OK = 0,
    BD_ERROR_INVALID_ARGUMENT = -1,
    BD_ERROR_CUDA = -2,
    BD_ERROR_OUT_OF_MEMORY = -3,
    BD_ERROR_NOT_SUPPORTED = -4,
    BD_ERROR_UNKNOWN = -5
} bd_status;

/*
 * Detector settings, 40 bytes (reference bdcudatag.h:54-65).  Fill with
 * bd_config_init() before changing fields.  max_hamming < 0 picks the family
 * default (2 for tag36h11, 1 for tag16h5; at most 3 is used); max_candidates
 * == 0 sizes the candidate cap from the frame area; max_detections is
 * clamped to [1, 256].
 */
typedef struct bd_config {
    uint32_t struct_size;
    int32_t max_hamming;
    int32_t min_cluster_pixels;
    int32_t min_tag_pixels;
    int32_t max_detections;
    int32_t max_candidates;
    int32_t refine_edges;
    int32_t use_cuda_graph;
    float min_decision_margin;
    float decode_sharpening;
} bd_config;

/*
 * One decoded tag, 84 bytes (reference bdcudatag.h:82-89).
 *   corners:    (x, y) pairs in pixel-index coordinates, starting at the
 *               tag's top-left corner and going top-right, bottom-right,
 *               bottom-left in the tag's canonical orientation.
 *   homography: row-major 3x3 map from the tag frame ([-1, 1]^2, x right,
 *               y down, first corner at (-1, -1)) to pixels,
 *               s * (px, py, 1)^T = H * (x, y, 1)^T, scaled so H[8] == 1.
 *   reserved:   always 0.
 */
typedef struct bd_detection {
    int32_t id;
    int32_t hamming;
    float decision_margin;
    float corners[8];
    int32_t reserved;
    float homography[9];
} bd_detection;

/* Per-detector counters of the most recent frame, 40 bytes (reference
 * bdcudatag.h:91-101). */
typedef struct bd_stats {
    uint64_t frames;
    float last_gpu_ms;
    float average_gpu_ms;
    float last_total_ms;
    int32_t runs;
    int32_t candidates;
    int32_t detections;
    int32_t quads;
    int32_t roi_rows;
} bd_stats;

BD_API uint32_t bd_api_version(void);
BD_API const char* bd_version_string(void);

BD_API int32_t bd_family_count(void);
BD_API const char* bd_family_name(int32_t family);
BD_API int32_t bd_family_bits_per_side(int32_t family);
BD_API int32_t bd_family_min_hamming(int32_t family);
BD_API int32_t bd_family_default_max_hamming(int32_t family);

BD_API void bd_config_init(bd_config* config);

/*
 * Creates a detector for one family and one frame size.  All device and
 * pinned host memory is allocated here; the detect calls never allocate.
 * On failure returns NULL, stores a bd_status in *status_out (when given)
 * and sets bd_last_error().  (reference bdcudatag.h:114-121)
 */
BD_API bd_detector* bd_detector_create(int32_t family, int32_t width, int32_t height,
                                       const bd_config* config, int32_t* status_out);
BD_API void bd_detector_destroy(bd_detector* detector);

/*
 * Detects tags in an 8-bit grayscale host image whose rows are `stride`
 * bytes apart (stride >= width).  Returns the number of tags found (after
 * de-duplication, at most max_detections) or a negative bd_status; writes
 * min(found, out_capacity) records, sorted by id.  (reference
 * bdcudatag.h:124-132)
 */
BD_API int32_t bd_detector_detect_host(bd_detector* detector, const uint8_t* gray,
                                       int32_t stride, bd_detection* out,
                                       int32_t out_capacity);

/*
 * Same as bd_detector_detect_host, for an image already in device memory of
 * the detector's CUDA context (no host-to-device copy).  The call does not
 * order itself after work on the caller's streams.  (reference
 * bdcudatag.h:134-140)
 */
BD_API int32_t bd_detector_detect_device(bd_detector* detector, const uint8_t* gray_device,
                                         int32_t stride, bd_detection* out,
                                         int32_t out_capacity);

BD_API void bd_detector_get_stats(bd_detector* detector, bd_stats* out);

/* Message of the latest failure on the calling thread (reference
 * bdcudatag.h:144-145). */
BD_API const char* bd_last_error(void);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
static_assert(sizeof(bd_config) == 40, "bd_config layout changed");
static_assert(sizeof(bd_detection) == 84, "bd_detection layout changed");
static_assert(sizeof(bd_stats) == 40, "bd_stats layout changed");
#endif

#endif /* BDCUDATAG_BDCUDATAG_H */
