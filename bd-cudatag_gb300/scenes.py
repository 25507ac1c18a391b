"""Seeded synthetic frames with ground truth (ctypes over libbdscenes.so).

Scene sets (the `scene_set` argument), with the benchmark workloads they feed:
  EIGHT_TAGS_640  640x480, 8 tag36h11 tags, side 40-120 px, noise sigma 4,
                  tilt <= 45 deg (the reference-style single-frame scenes)
  MIXED_1280      1280x800, 6 tag36h11 + 2 tag16h5, side 20-200 px, sigma 6,
                  blur on odd frames, two decoys on frames i % 4 == 3, glyph
                  clutter past the candidate cap on i % 8 == 5
  MULTI_SIZE      any size, 4-24 tags of both families, side 16-300 px,
                  sigma 2-8 (16-frame batches of uneven sizes)
  REFINE_1280     as MIXED_1280, own seeds (corner-refinement quads)
  SERVING         0-40 tags, 10% blank frames, sigma 2-8 (camera streams)
Set k uses base seed 6324 + 1000*k and frame i uses seed base + i.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from pathlib import Path

import numpy as np

_LIB = None
MAX_TAGS = 64
EIGHT_TAGS_640, MIXED_1280, MULTI_SIZE, REFINE_1280, SERVING = 1, 2, 3, 4, 5


def base_seed(scene_set: int) -> int:
    return 6324 + 1000 * scene_set


class _Tag(ctypes.Structure):
    _fields_ = [("family", ctypes.c_int32), ("id", ctypes.c_int32), ("corners", ctypes.c_double * 8)]


def lib() -> ctypes.CDLL:
    global _LIB
    if _LIB is None:
        path = Path(__file__).resolve().parent / "libbdscenes.so"
        if not path.exists():
            raise RuntimeError(f"{path} is not built; run __graft_entry__.build()")
        _LIB = ctypes.CDLL(str(path))
        _LIB.bds_make_pose.argtypes = [ctypes.c_double] * 5 + [ctypes.POINTER(ctypes.c_double)]
        _LIB.bds_render_tag.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                        ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p]
        _LIB.bds_ref_scenes.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint32,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _LIB.bds_render_scene.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_int]
        _LIB.bds_render_many.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_int]
    return _LIB


def make_pose(cx: float, cy: float, size: float, angle: float, perspective: float = 0.0) -> np.ndarray:
    out = (ctypes.c_double * 9)()
    lib().bds_make_pose(cx, cy, size, angle, perspective, out)
    return np.array(out, dtype=np.float64)


def project(pose: np.ndarray, x: float, y: float) -> tuple[float, float]:
    v = pose
    w = v[6] * x + v[7] * y + v[8]
    return (v[0] * x + v[1] * y + v[2]) / w, (v[3] * x + v[4] * y + v[5]) / w


def render_tag(family: int, tag_id: int, width: int, height: int, pose: np.ndarray,
               supersample: int = 2, code: int | None = None, flip_one_bit: bool = False) -> np.ndarray:
    img = np.empty((height, width), dtype=np.uint8)
    p = np.ascontiguousarray(pose, dtype=np.float64)
    rc = lib().bds_render_tag(family, tag_id, width, height,
                              p.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), supersample,
                              0 if code is None else code, 0 if code is None else 1,
                              1 if flip_one_bit else 0, img.ctypes.data)
    if rc != 0:
        raise ValueError("bad render_tag arguments")
    return img


def ref_scenes(width: int, height: int, count: int = 32, seed: int = 6324):
    """The reference benchmark scene set: (images[count,H,W], ids[count,8], corners[count,8,4,2])."""
    images = np.empty((count, height, width), dtype=np.uint8)
    ids = np.empty((count, 8), dtype=np.int32)
    corners = np.empty((count, 8, 4, 2), dtype=np.float64)
    lib().bds_ref_scenes(width, height, count, seed, images.ctypes.data, ids.ctypes.data,
                         corners.ctypes.data)
    return images, ids, corners


@dataclass
class TagTruth:
    family: int
    id: int
    corners: np.ndarray  # (4, 2), pixel-index convention


def render_scene(scene_set: int, index: int, width: int, height: int,
                  seed: int | None = None) -> tuple[np.ndarray, list[TagTruth]]:
    img = np.empty((height, width), dtype=np.uint8)
    tags = (_Tag * MAX_TAGS)()
    s = base_seed(scene_set) + index if seed is None else seed
    n = lib().bds_render_scene(scene_set, s, index, width, height, img.ctypes.data, tags, MAX_TAGS)
    truth = [TagTruth(tags[i].family, tags[i].id, np.array(tags[i].corners).reshape(4, 2))
             for i in range(n)]
    return img, truth


def render_many(scene_set: int, sizes: list[tuple[int, int]], threads: int = 8,
                base: int | None = None):
    """Renders len(sizes) frames (frame i with seed base + i) on host threads.

    Returns (list of HxW uint8 arrays viewing one packed buffer, tag counts,
    tag records array).
    """
    count = len(sizes)
    widths = np.array([w for w, _ in sizes], dtype=np.int32)
    heights = np.array([h for _, h in sizes], dtype=np.int32)
    total = int(np.sum(widths.astype(np.int64) * heights))
    packed = np.empty(total, dtype=np.uint8)
    tags = (_Tag * (MAX_TAGS * count))()
    counts = np.zeros(count, dtype=np.int32)
    b = base_seed(scene_set) if base is None else base
    lib().bds_render_many(scene_set, b, count, widths.ctypes.data, heights.ctypes.data,
                          packed.ctypes.data, tags, MAX_TAGS, counts.ctypes.data, threads)
    frames = []
    off = 0
    for w, h in sizes:
        frames.append(packed[off:off + w * h].reshape(h, w))
        off += w * h
    truth = []
    for i in range(count):
        truth.append([TagTruth(tags[i * MAX_TAGS + k].family, tags[i * MAX_TAGS + k].id,
                               np.array(tags[i * MAX_TAGS + k].corners).reshape(4, 2))
                      for k in range(counts[i])])
    return frames, truth
