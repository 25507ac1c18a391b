"""ctypes binding of libbdcudatag.so (the GB300 detector library).

The structure mirrors and the function signatures are those of the
reference's own ctypes consumer (detector/bench/compare_detectors.py:76-156),
so code written against the reference binds this library unchanged; the
batch entry points of bdcudatag_gb300.h are added.

Loading fails loudly when the library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libbdcudatag.so"

FAMILY_TAG36H11 = 0
FAMILY_TAG16H5 = 1
OK = 0
ERROR_INVALID_ARGUMENT = -1
ERROR_CUDA = -2
ERROR_OUT_OF_MEMORY = -3
ERROR_NOT_SUPPORTED = -4
ERROR_UNKNOWN = -5


class Config(ctypes.Structure):
    _fields_ = [
        ("struct_size", ctypes.c_uint32),
        ("max_hamming", ctypes.c_int32),
        ("min_cluster_pixels", ctypes.c_int32),
        ("min_tag_pixels", ctypes.c_int32),
        ("max_detections", ctypes.c_int32),
        ("max_candidates", ctypes.c_int32),
        ("refine_edges", ctypes.c_int32),
        ("use_cuda_graph", ctypes.c_int32),
        ("min_decision_margin", ctypes.c_float),
        ("decode_sharpening", ctypes.c_float),
    ]


class Stats(ctypes.Structure):
    _fields_ = [
        ("frames", ctypes.c_uint64),
        ("last_gpu_ms", ctypes.c_float),
        ("average_gpu_ms", ctypes.c_float),
        ("last_total_ms", ctypes.c_float),
        ("runs", ctypes.c_int32),
        ("candidates", ctypes.c_int32),
        ("detections", ctypes.c_int32),
        ("quads", ctypes.c_int32),
        ("roi_rows", ctypes.c_int32),
    ]


class Detection(ctypes.Structure):
    _fields_ = [
        ("id", ctypes.c_int32),
        ("hamming", ctypes.c_int32),
        ("decision_margin", ctypes.c_float),
        ("corners", ctypes.c_float * 8),
        ("reserved", ctypes.c_int32),
        ("homography", ctypes.c_float * 9),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("rejected", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("mean_batch_frames", ctypes.c_double), ("plans", ctypes.c_int32),
                ("peak_inflight", ctypes.c_int32), ("device_bytes", ctypes.c_int64)]


class RefineArgs(ctypes.Structure):
    _fields_ = [("images", ctypes.c_void_p), ("image_pitch", ctypes.c_int64),
                ("width", ctypes.c_int32), ("height", ctypes.c_int32), ("stride", ctypes.c_int32),
                ("count", ctypes.c_int32), ("image_index", ctypes.c_void_p),
                ("corners", ctypes.c_void_p), ("templates", ctypes.c_void_p),
                ("levels", ctypes.c_void_p), ("cells", ctypes.c_int32),
                ("samples_per_cell", ctypes.c_int32)]


class LaunchConfig(ctypes.Structure):
    _fields_ = [("stats_rows", ctypes.c_int32), ("quad_warps", ctypes.c_int32),
                ("quad_ctas_per_sm", ctypes.c_int32), ("quad_split", ctypes.c_int32),
                ("band_cap", ctypes.c_int32), ("fit_merged", ctypes.c_int32),
                ("persistent", ctypes.c_int32),
                ("persist_ctas", ctypes.c_int32)]


class Camera(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("families", ctypes.c_uint32), ("reserved", ctypes.c_int32)]


DETECTION_DTYPE = np.dtype([("id", "<i4"), ("hamming", "<i4"), ("decision_margin", "<f4"),
                            ("corners", "<f4", (8,)), ("reserved", "<i4"),
                            ("homography", "<f4", (9,))])
assert DETECTION_DTYPE.itemsize == ctypes.sizeof(Detection) == 84
assert ctypes.sizeof(Config) == 40 and ctypes.sizeof(Stats) == 40 and ctypes.sizeof(Camera) == 16

# Every C symbol the library exports (include/bdcudatag/*.h).
REFERENCE_SYMBOLS = [
    "bd_api_version", "bd_version_string", "bd_family_count", "bd_family_name",
    "bd_family_bits_per_side", "bd_family_min_hamming", "bd_family_default_max_hamming",
    "bd_config_init", "bd_detector_create", "bd_detector_destroy", "bd_detector_detect_host",
    "bd_detector_detect_device", "bd_detector_get_stats", "bd_last_error",
]
GB300_SYMBOLS = [
    "bd_batch_create", "bd_batch_destroy", "bd_batch_camera_count", "bd_batch_max_detections",
    "bd_batch_device_bytes", "bd_batch_detect_host", "bd_batch_detect_device",
    "bd_batch_submit_host", "bd_batch_submit_device", "bd_batch_wait", "bd_batch_host_frame",
    "bd_batch_last_gpu_ms", "bd_batch_counts", "bd_batch_debug_stage", "bd_detector_debug_stage",
    "bd_batch_set_stream", "bd_stage_count", "bd_stage_name", "bd_batch_profile_device",
    "bd_batch_query", "bd_tile_stats_device_noalloc",
    "bd_server_create", "bd_server_destroy", "bd_server_submit", "bd_server_wait",
    "bd_server_poll", "bd_server_get_stats",
    "bd_tag_template", "bd_refine_forward", "bd_refine_backward", "bd_refine_gauss_newton",
    "bd_batch_get_launch", "bd_batch_set_launch", "bd_batch_autotune", "bd_batch_pipeline",
    "bd_batch_debug_persist",
]

_LIB = None
_P = ctypes.c_void_p


def lib() -> ctypes.CDLL:
    """The detector library (libbdcudatag.so next to this file), bound."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
        _LIB = load(LIB_PATH)
    return _LIB


def load(path) -> ctypes.CDLL:
    """Loads and binds a build of the library at `path` (for example the
    reference-arithmetic variant that build.py makes for a test).  Every load
    has its own symbols and its own CUDA kernels."""
    L = ctypes.CDLL(str(path))
    L.bd_api_version.restype = ctypes.c_uint32
    L.bd_version_string.restype = ctypes.c_char_p
    L.bd_family_name.restype = ctypes.c_char_p
    L.bd_family_name.argtypes = [ctypes.c_int32]
    for n in ("bd_family_bits_per_side", "bd_family_min_hamming", "bd_family_default_max_hamming"):
        getattr(L, n).argtypes = [ctypes.c_int32]
        getattr(L, n).restype = ctypes.c_int32
    L.bd_config_init.argtypes = [ctypes.POINTER(Config)]
    L.bd_detector_create.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                     ctypes.POINTER(Config), ctypes.POINTER(ctypes.c_int32)]
    L.bd_detector_create.restype = _P
    L.bd_detector_destroy.argtypes = [_P]
    for n in ("bd_detector_detect_host", "bd_detector_detect_device"):
        getattr(L, n).argtypes = [_P, _P, ctypes.c_int32, _P, ctypes.c_int32]
        getattr(L, n).restype = ctypes.c_int32
    L.bd_detector_get_stats.argtypes = [_P, ctypes.POINTER(Stats)]
    L.bd_last_error.restype = ctypes.c_char_p
    L.bd_batch_create.argtypes = [_P, ctypes.c_int32, ctypes.POINTER(Config),
                                  ctypes.POINTER(ctypes.c_int32)]
    L.bd_batch_create.restype = _P
    L.bd_batch_destroy.argtypes = [_P]
    L.bd_batch_camera_count.argtypes = [_P]
    L.bd_batch_max_detections.argtypes = [_P]
    L.bd_batch_device_bytes.argtypes = [_P]
    L.bd_batch_device_bytes.restype = ctypes.c_int64
    for n in ("bd_batch_detect_host", "bd_batch_detect_device"):
        getattr(L, n).argtypes = [_P, _P, _P, _P, _P]
        getattr(L, n).restype = ctypes.c_int32
    for n in ("bd_batch_submit_host", "bd_batch_submit_device"):
        getattr(L, n).argtypes = [_P, _P, _P]
        getattr(L, n).restype = ctypes.c_int32
    L.bd_batch_wait.argtypes = [_P, _P, _P]
    L.bd_batch_wait.restype = ctypes.c_int32
    L.bd_batch_host_frame.argtypes = [_P, ctypes.c_int32]
    L.bd_batch_host_frame.restype = _P
    L.bd_batch_last_gpu_ms.argtypes = [_P]
    L.bd_batch_last_gpu_ms.restype = ctypes.c_float
    L.bd_batch_counts.argtypes = [_P, ctypes.c_int32, _P]
    L.bd_batch_debug_stage.argtypes = [_P, ctypes.c_int32, ctypes.c_char_p, _P, ctypes.c_int64]
    L.bd_batch_debug_stage.restype = ctypes.c_int64
    L.bd_detector_debug_stage.argtypes = [_P, ctypes.c_char_p, _P, ctypes.c_int64]
    L.bd_detector_debug_stage.restype = ctypes.c_int64
    L.bd_batch_set_stream.argtypes = [_P, _P]
    L.bd_stage_name.restype = ctypes.c_char_p
    L.bd_stage_name.argtypes = [ctypes.c_int32]
    L.bd_batch_profile_device.argtypes = [_P, _P, _P, _P]
    L.bd_batch_query.argtypes = [_P]
    L.bd_tile_stats_device_noalloc.argtypes = [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                               _P, _P, _P, _P]
    L.bd_tile_stats_device_noalloc.restype = ctypes.c_int32
    L.bd_server_create.argtypes = [_P, ctypes.c_int32, ctypes.POINTER(Config), ctypes.c_int64,
                                   ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]
    L.bd_server_create.restype = _P
    L.bd_server_destroy.argtypes = [_P]
    L.bd_server_submit.argtypes = [_P, ctypes.c_int32, _P, ctypes.c_int32]
    L.bd_server_submit.restype = ctypes.c_int64
    for n in ("bd_server_wait", "bd_server_poll"):
        getattr(L, n).argtypes = [_P, ctypes.c_int64, _P, _P, ctypes.POINTER(ctypes.c_double)]
        getattr(L, n).restype = ctypes.c_int32
    L.bd_server_get_stats.argtypes = [_P, ctypes.POINTER(ServerStats)]
    L.bd_batch_get_launch.argtypes = [_P, ctypes.POINTER(LaunchConfig)]
    L.bd_batch_set_launch.argtypes = [_P, ctypes.POINTER(LaunchConfig)]
    L.bd_batch_debug_persist.argtypes = [_P, ctypes.c_int64, ctypes.c_int32]
    L.bd_batch_set_launch.restype = ctypes.c_int32
    L.bd_batch_autotune.argtypes = [_P, _P, _P, ctypes.c_int32, ctypes.POINTER(LaunchConfig),
                                    ctypes.POINTER(ctypes.c_float)]
    L.bd_batch_autotune.restype = ctypes.c_int32
    L.bd_batch_pipeline.argtypes = [_P, ctypes.c_int32, _P, _P, ctypes.c_int32, ctypes.c_int32,
                                    ctypes.c_int32, _P, ctypes.POINTER(ctypes.c_double)]
    L.bd_batch_pipeline.restype = ctypes.c_int32
    L.bd_tag_template.argtypes = [ctypes.c_int32, ctypes.c_int32, _P]
    L.bd_tag_template.restype = ctypes.c_int32
    L.bd_refine_forward.argtypes = [ctypes.POINTER(RefineArgs), _P, _P, _P]
    L.bd_refine_forward.restype = ctypes.c_int32
    L.bd_refine_backward.argtypes = [ctypes.POINTER(RefineArgs), _P, _P, _P, _P]
    L.bd_refine_backward.restype = ctypes.c_int32
    L.bd_refine_gauss_newton.argtypes = [ctypes.POINTER(RefineArgs), _P, ctypes.c_int32, _P, _P]
    L.bd_refine_gauss_newton.restype = ctypes.c_int32
    L.bd_batch_query.restype = ctypes.c_int32
    return L


def default_config(**overrides) -> Config:
    c = Config()
    lib().bd_config_init(ctypes.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def last_error() -> str:
    msg = lib().bd_last_error()
    return msg.decode() if msg else ""


def _ptr(x) -> int:
    """Address of a numpy array, a torch tensor (host or device) or an int."""
    if isinstance(x, int):
        return x
    if hasattr(x, "data_ptr"):
        return x.data_ptr()
    return x.ctypes.data


_STAGE_DTYPES = {
    "tile_min": np.uint8, "tile_max": np.uint8, "bits": np.uint32, "row_count": np.uint32,
    "runs": np.uint32, "label": np.uint32, "area": np.uint32, "bbox": np.uint32,
    "candidates": np.uint32, "hull_quads": np.float32, "quads": np.float32,
    "decodes": np.dtype([("id", "<i4"), ("hamming", "<i4"), ("margin", "<f4"), ("corners", "<f4", (8,))]),
    "state": np.uint32,
}


def _stage(fn, *args, name: str) -> np.ndarray:
    size = fn(*args, name.encode(), None, 0)
    if size < 0:
        raise KeyError(name)
    dt = np.dtype(_STAGE_DTYPES[name])
    out = np.zeros(size // dt.itemsize, dtype=dt)
    fn(*args, name.encode(), out.ctypes.data, size)
    return out


class Detector:
    """One family, one frame size: the reference's bd_detector."""

    def __init__(self, family: int, width: int, height: int, config: Config | None = None,
                 library: ctypes.CDLL | None = None):
        """library: a build loaded with load() (default: the library)."""
        self._L = library if library is not None else lib()
        status = ctypes.c_int32(0)
        cfg = config if config is not None else default_config()
        self.handle = self._L.bd_detector_create(family, width, height, ctypes.byref(cfg),
                                                 ctypes.byref(status))
        if not self.handle:
            raise RuntimeError(f"bd_detector_create failed ({status.value}): {last_error()}")
        self.family, self.width, self.height = family, width, height
        self.max_detections = min(max(cfg.max_detections, 1), 256)
        self.out = np.zeros(self.max_detections, dtype=DETECTION_DTYPE)

    def detect(self, gray: np.ndarray, stride: int | None = None, capacity: int | None = None):
        """Returns (found, detections written)."""
        cap = self.max_detections if capacity is None else capacity
        s = gray.strides[0] if stride is None else stride
        n = self._L.bd_detector_detect_host(self.handle, _ptr(gray), s, self.out.ctypes.data, cap)
        if n < 0:
            raise RuntimeError(f"detect failed ({n}): {last_error()}")
        return n, self.out[:min(n, cap)].copy()

    def detect_device(self, gray_device, stride: int, capacity: int | None = None):
        cap = self.max_detections if capacity is None else capacity
        n = self._L.bd_detector_detect_device(self.handle, _ptr(gray_device), stride,
                                            self.out.ctypes.data, cap)
        if n < 0:
            raise RuntimeError(f"detect_device failed ({n}): {last_error()}")
        return n, self.out[:min(n, cap)].copy()

    def stats(self) -> Stats:
        s = Stats()
        self._L.bd_detector_get_stats(self.handle, ctypes.byref(s))
        return s

    def stage(self, name: str) -> np.ndarray:
        return _stage(self._L.bd_detector_debug_stage, self.handle, name=name)

    def close(self) -> None:
        if getattr(self, "handle", None):
            self._L.bd_detector_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


class Batch:
    """A fixed set of cameras detected together (bd_batch)."""

    def __init__(self, cameras: list[tuple[int, int, int]], config: Config | None = None):
        arr = (Camera * len(cameras))(*[Camera(w, h, fam, 0) for w, h, fam in cameras])
        status = ctypes.c_int32(0)
        cfg = config if config is not None else default_config()
        self.handle = lib().bd_batch_create(ctypes.cast(arr, _P), len(cameras), ctypes.byref(cfg),
                                            ctypes.byref(status))
        if not self.handle:
            raise RuntimeError(f"bd_batch_create failed ({status.value}): {last_error()}")
        self.cameras = list(cameras)
        self.n = len(cameras)
        self.max_detections = lib().bd_batch_max_detections(self.handle)
        self.out = np.zeros((self.n, 2, self.max_detections), dtype=DETECTION_DTYPE)
        self.found = np.zeros((self.n, 2), dtype=np.int32)
        self._ptrs = (ctypes.c_void_p * self.n)()
        self._strides = np.zeros(self.n, dtype=np.int32)

    def _set(self, frames, strides):
        for i, f in enumerate(frames):
            self._ptrs[i] = _ptr(f)
            self._strides[i] = strides[i] if strides is not None else \
                (f.strides[0] if hasattr(f, "strides") and not hasattr(f, "data_ptr") else self.cameras[i][0])

    def detect(self, frames, strides=None, device: bool = False):
        self._set(frames, strides)
        fn = lib().bd_batch_detect_device if device else lib().bd_batch_detect_host
        rc = fn(self.handle, ctypes.cast(self._ptrs, _P), self._strides.ctypes.data,
                self.out.ctypes.data, self.found.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"batch detect failed ({rc}): {last_error()}")
        return self.found.copy(), self.out.copy()

    def submit(self, frames, strides=None, device: bool = False) -> None:
        self._set(frames, strides)
        fn = lib().bd_batch_submit_device if device else lib().bd_batch_submit_host
        rc = fn(self.handle, ctypes.cast(self._ptrs, _P), self._strides.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"batch submit failed ({rc}): {last_error()}")

    def wait(self, copy: bool = True):
        rc = lib().bd_batch_wait(self.handle, self.out.ctypes.data, self.found.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"batch wait failed ({rc}): {last_error()}")
        return (self.found.copy(), self.out.copy()) if copy else (self.found, self.out)

    def set_stream(self, stream) -> None:
        """stream: a torch.cuda.Stream, an int handle or None."""
        handle = 0 if stream is None else (stream.cuda_stream if hasattr(stream, "cuda_stream") else int(stream))
        lib().bd_batch_set_stream(self.handle, handle or None)

    def profile_device(self, frames, strides=None) -> dict:
        self._set(frames, strides)
        n = lib().bd_stage_count()
        ms = np.zeros(n, dtype=np.float32)
        rc = lib().bd_batch_profile_device(self.handle, ctypes.cast(self._ptrs, _P),
                                           self._strides.ctypes.data, ms.ctypes.data)
        if rc != 0:
            raise RuntimeError(f"profile failed ({rc}): {last_error()}")
        return {lib().bd_stage_name(i).decode(): float(ms[i]) for i in range(n)}

    def query(self) -> bool:
        r = lib().bd_batch_query(self.handle)
        if r < 0:
            raise RuntimeError(f"batch query failed ({r}): {last_error()}")
        return r == 1

    def launch(self) -> dict:
        lc = LaunchConfig()
        lib().bd_batch_get_launch(self.handle, ctypes.byref(lc))
        return {f: getattr(lc, f) for f, _ in LaunchConfig._fields_}

    def set_launch(self, **fields) -> None:
        lc = LaunchConfig()
        lib().bd_batch_get_launch(self.handle, ctypes.byref(lc))
        for k, v in fields.items():
            setattr(lc, k, v)
        rc = lib().bd_batch_set_launch(self.handle, ctypes.byref(lc))
        if rc != 0:
            raise RuntimeError(f"set_launch failed ({rc}): {last_error()}")

    def debug_persist(self, timeout_ns: int = 1_000_000_000, stall_frame: int = -1) -> None:
        """Test hook of the persistent launch (bd_batch_debug_persist)."""
        rc = lib().bd_batch_debug_persist(self.handle, int(timeout_ns), int(stall_frame))
        if rc != 0:
            raise RuntimeError(f"debug_persist failed ({rc}): {last_error()}")

    def autotune(self, frames_device, strides=None, iterations: int = 20):
        self._set(frames_device, strides)
        lc = LaunchConfig()
        ms = ctypes.c_float(0.0)
        rc = lib().bd_batch_autotune(self.handle, ctypes.cast(self._ptrs, _P),
                                     self._strides.ctypes.data, iterations, ctypes.byref(lc),
                                     ctypes.byref(ms))
        if rc != 0:
            raise RuntimeError(f"autotune failed ({rc}): {last_error()}")
        return {f: getattr(lc, f) for f, _ in LaunchConfig._fields_}, ms.value

    def host_frame(self, i: int) -> np.ndarray:
        w, h, _ = self.cameras[i]
        p = lib().bd_batch_host_frame(self.handle, i)
        return np.ctypeslib.as_array((ctypes.c_uint8 * (w * h)).from_address(p)).reshape(h, w)

    def counts(self, i: int) -> np.ndarray:
        c = np.zeros(5, dtype=np.uint32)
        lib().bd_batch_counts(self.handle, i, c.ctypes.data)
        return c

    def last_gpu_ms(self) -> float:
        return lib().bd_batch_last_gpu_ms(self.handle)

    def device_bytes(self) -> int:
        return lib().bd_batch_device_bytes(self.handle)

    def stage(self, camera: int, name: str) -> np.ndarray:
        return _stage(lib().bd_batch_debug_stage, self.handle, camera, name=name)

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().bd_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


class Server:
    """Continuous-batching server over several cameras (bd_server)."""

    def __init__(self, cameras: list[tuple[int, int, int]], config: Config | None = None,
                 device_budget: int = 8 << 30, max_batches: int = 4, queue_depth: int = 8):
        arr = (Camera * len(cameras))(*[Camera(w, h, fam, 0) for w, h, fam in cameras])
        status = ctypes.c_int32(0)
        cfg = config if config is not None else default_config()
        self.handle = lib().bd_server_create(ctypes.cast(arr, _P), len(cameras), ctypes.byref(cfg),
                                             device_budget, max_batches, queue_depth,
                                             ctypes.byref(status))
        if not self.handle:
            raise RuntimeError(f"bd_server_create failed ({status.value}): {last_error()}")
        self.cameras = list(cameras)
        self.max_detections = min(max(cfg.max_detections, 1), 256)

    def submit(self, camera: int, frame, stride: int | None = None) -> int:
        s = stride if stride is not None else self.cameras[camera][0]
        t = lib().bd_server_submit(self.handle, camera, _ptr(frame), s)
        return int(t)

    def wait(self, ticket: int, block: bool = True):
        """(status, found[2], detections[2, max_detections], latency_ms)."""
        out = np.zeros((2, self.max_detections), dtype=DETECTION_DTYPE)
        found = np.zeros(2, dtype=np.int32)
        lat = ctypes.c_double(0.0)
        fn = lib().bd_server_wait if block else lib().bd_server_poll
        rc = fn(self.handle, ticket, out.ctypes.data, found.ctypes.data, ctypes.byref(lat))
        if rc < 0:
            raise RuntimeError(f"server wait failed ({rc}): {last_error()}")
        return rc, found, out, lat.value

    def stats(self) -> ServerStats:
        st = ServerStats()
        lib().bd_server_get_stats(self.handle, ctypes.byref(st))
        return st

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().bd_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        self.close()


def tag_template(family: int, tag_id: int) -> np.ndarray:
    """(cells, cells) uint8 template of a tag, 1 = white (quiet zone included)."""
    cells = 10 if family == 0 else 8
    out = np.zeros(cells * cells, dtype=np.uint8)
    n = lib().bd_tag_template(family, tag_id, out.ctypes.data)
    if n < 0:
        raise ValueError("bad family or id")
    return out.reshape(cells, cells)


def refine_args(images, corners, templates, image_index=None, levels=None,
                samples_per_cell: int = 8) -> RefineArgs:
    """Arguments over torch CUDA tensors: images [F, H, W] uint8, corners
    [n, 8] float32, templates [n, cells, cells] uint8, image_index [n] int32,
    levels [n, 2] float32."""
    f, h, w = images.shape
    return RefineArgs(images.data_ptr(), h * images.stride(1), w, h, images.stride(1),
                      corners.shape[0], image_index.data_ptr() if image_index is not None else None,
                      corners.data_ptr(), templates.data_ptr(),
                      levels.data_ptr() if levels is not None else None, templates.shape[-1],
                      samples_per_cell)


def pipeline(batches: list, frame_sets: list, strides, steps: int, device: bool = True):
    """Runs `steps` batches round-robin over `batches` in native code.
    frame_sets: list of per-camera frame lists.  Returns (wall ms, per-batch
    latency ms array)."""
    cams = len(frame_sets[0])
    handles = (ctypes.c_void_p * len(batches))(*[b.handle for b in batches])
    flat = (ctypes.c_void_p * (cams * len(frame_sets)))(*[_ptr(f) for fs in frame_sets for f in fs])
    st = np.asarray(strides, dtype=np.int32)
    lat = np.zeros(max(steps, 1), dtype=np.float32)
    wall = ctypes.c_double(0.0)
    rc = lib().bd_batch_pipeline(ctypes.cast(handles, _P), len(batches), ctypes.cast(flat, _P),
                                 st.ctypes.data, len(frame_sets), steps, 1 if device else 0,
                                 lat.ctypes.data, ctypes.byref(wall))
    if rc != 0:
        raise RuntimeError(f"pipeline failed ({rc}): {last_error()}")
    return wall.value, lat[:steps]
