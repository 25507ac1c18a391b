"""CPU ORACLE -- test infrastructure, not part of the product.

ctypes binding of oracle/_build/liboracle.so, the sequential C++
restatement of the reference pipeline (see oracle/oracle.h for what it
restates and how it is pinned).  Only tests/, the smoke check and the CPU
baseline of bench.py use it.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
# The same restatement built with multiply-add contraction (as nvcc builds the
# reference): only the rounding-sensitivity test uses it.
LIB_FMA_PATH = HERE / "_build" / "liboracle_fma.so"
_LIBS: dict = {}


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


class Detection(ctypes.Structure):
    _fields_ = [
        ("id", ctypes.c_int32),
        ("hamming", ctypes.c_int32),
        ("decision_margin", ctypes.c_float),
        ("corners", ctypes.c_float * 8),
        ("reserved", ctypes.c_int32),
        ("homography", ctypes.c_float * 9),
    ]


DETECTION_DTYPE = np.dtype([("id", "<i4"), ("hamming", "<i4"), ("decision_margin", "<f4"),
                            ("corners", "<f4", (8,)), ("reserved", "<i4"),
                            ("homography", "<f4", (9,))])
DECODE_DTYPE = np.dtype([("id", "<i4"), ("hamming", "<i4"), ("margin", "<f4"),
                         ("corners", "<f4", (8,))])


def default_config(**overrides) -> Config:
    c = Config(40, -1, 24, 8, 64, 0, 1, 1, 3.0, 0.25)
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def build() -> Path:
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB_PATH


def lib(fma: bool = False) -> ctypes.CDLL:
    if fma not in _LIBS:
        path = LIB_FMA_PATH if fma else LIB_PATH
        if not path.exists():
            build()
        L = ctypes.CDLL(str(path))
        L.bdo_run.restype = ctypes.c_void_p
        L.bdo_run.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                              ctypes.c_int32, ctypes.POINTER(Config)]
        L.bdo_free.argtypes = [ctypes.c_void_p]
        L.bdo_detections.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
        L.bdo_detections.restype = ctypes.c_int32
        L.bdo_counts.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.bdo_geometry.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.bdo_stage.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        L.bdo_stage.restype = ctypes.c_int64
        L.bdo_detect_many.argtypes = [ctypes.c_int32] + [ctypes.c_void_p] * 5 + \
            [ctypes.POINTER(Config), ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
             ctypes.c_void_p]
        L.bdo_detect_many.restype = ctypes.c_int32
        L.bdo_refit64.argtypes = [ctypes.c_void_p] * 4
        L.bdo_refit64.restype = ctypes.c_int32
        L.bdo_homography64.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        for name in ("bdo_sinf", "bdo_cosf"):
            getattr(L, name).argtypes = [ctypes.c_float]
            getattr(L, name).restype = ctypes.c_float
        L.bdo_atan2f.argtypes = [ctypes.c_float, ctypes.c_float]
        L.bdo_atan2f.restype = ctypes.c_float
        _LIBS[fma] = L
    return _LIBS[fma]


_STAGE_DTYPES = {
    "tile_min": np.uint8, "tile_max": np.uint8, "tile_mean": np.uint8, "thresh": np.uint8,
    "active": np.uint8, "span_hist": np.uint32, "mean_hist": np.uint32, "ref": np.uint32,
    "row_active": np.uint8, "row_start": np.int32, "row_end": np.int32, "bits": np.uint32,
    "row_count": np.uint32, "runs": np.uint32, "label": np.uint32, "area": np.uint32,
    "bbox": np.uint32, "candidates": np.uint32, "hull_quads": np.float32, "quads": np.float32,
    "decodes": DECODE_DTYPE,
}


class Frame:
    """One frame run through the oracle; stage buffers on demand."""

    def __init__(self, gray: np.ndarray, family: int = 0, config: Config | None = None,
                 stride: int | None = None, fma: bool = False):
        gray = np.ascontiguousarray(gray, dtype=np.uint8) if stride is None else gray
        h, w = gray.shape[0], (gray.shape[1] if stride is None else None)
        if stride is None:
            stride = gray.shape[1]
        else:
            w = gray.shape[1] if w is None else w
        self.width, self.height, self.family = int(w), int(h), family
        cfg = config if config is not None else default_config()
        self._lib = lib(fma)
        self._h = self._lib.bdo_run(gray.ctypes.data, self.width, self.height, stride, family,
                                ctypes.byref(cfg))
        if not self._h:
            raise ValueError("oracle rejected the frame")
        g = (ctypes.c_int32 * 9)()
        self._lib.bdo_geometry(self._h, g)
        (self.tile_w, self.tile_h, self.words, self.row_cap, self.max_candidates,
         self.max_detections, self.dim, self.max_hamming, self.candidate_count) = list(g)

    def __del__(self):
        if getattr(self, "_h", None):
            self._lib.bdo_free(self._h)
            self._h = None

    def detections(self, capacity: int | None = None) -> tuple[int, np.ndarray]:
        cap = self.max_detections if capacity is None else capacity
        out = np.zeros(max(cap, 1), dtype=DETECTION_DTYPE)
        found = self._lib.bdo_detections(self._h, out.ctypes.data, cap)
        return found, out[:min(found, cap)]

    def counts(self) -> np.ndarray:
        c = np.zeros(5, dtype=np.uint32)
        self._lib.bdo_counts(self._h, c.ctypes.data)
        return c

    def refit64(self, gray: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """FP64 re-fit of every candidate: (hull quads, refined quads), each
        float64[candidate_count, 8] with NaN rows where no quad was fitted.
        `gray` must be the image this frame was run on."""
        n = self.candidate_count
        hq = np.full((max(n, 1), 8), np.nan)
        q = np.full((max(n, 1), 8), np.nan)
        img = np.ascontiguousarray(gray, dtype=np.uint8)
        assert img.shape == (self.height, self.width)
        self._lib.bdo_refit64(self._h, img.ctypes.data, hq.ctypes.data, q.ctypes.data)
        return hq[:n], q[:n]

    def stage(self, name: str) -> np.ndarray:
        size = self._lib.bdo_stage(self._h, name.encode(), None, 0)
        if size < 0:
            raise KeyError(name)
        dt = np.dtype(_STAGE_DTYPES[name])
        out = np.zeros(size // dt.itemsize, dtype=dt)
        self._lib.bdo_stage(self._h, name.encode(), out.ctypes.data, size)
        return out


def homography64(corners: np.ndarray) -> np.ndarray:
    """The result-record homography from FP64 corners, in FP64 (float64[9])."""
    c = np.ascontiguousarray(corners, dtype=np.float64).reshape(8)
    h = np.zeros(9, dtype=np.float64)
    lib().bdo_homography64(c.ctypes.data, h.ctypes.data)
    return h


def detect(gray: np.ndarray, family: int = 0, config: Config | None = None) -> np.ndarray:
    found, dets = Frame(gray, family, config).detections()
    return dets


def detect_many(frames: list[np.ndarray], family_masks: list[int], config: Config | None = None,
                threads: int = 1, max_detections: int = 64):
    n = len(frames)
    ptrs = (ctypes.c_void_p * n)(*[f.ctypes.data for f in frames])
    widths = np.array([f.shape[1] for f in frames], dtype=np.int32)
    heights = np.array([f.shape[0] for f in frames], dtype=np.int32)
    strides = widths.copy()
    masks = np.array(family_masks, dtype=np.uint32)
    out = np.zeros(n * 2 * max_detections, dtype=DETECTION_DTYPE)
    counts = np.zeros(n * 2, dtype=np.int32)
    cfg = config if config is not None else default_config(max_detections=max_detections)
    rc = lib().bdo_detect_many(n, ptrs, widths.ctypes.data, heights.ctypes.data,
                               strides.ctypes.data, masks.ctypes.data, ctypes.byref(cfg), threads,
                               out.ctypes.data, max_detections, counts.ctypes.data)
    if rc != 0:
        raise RuntimeError("bdo_detect_many failed")
    return out.reshape(n, 2, max_detections), counts.reshape(n, 2)
