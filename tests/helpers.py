"""Shared test helpers: ground truth, matching and the reference KAT scenes."""
from __future__ import annotations

import itertools

import numpy as np

import scenes

UNIT = [(-1.0, -1.0), (1.0, -1.0), (1.0, 1.0), (-1.0, 1.0)]


def pose_corners(pose) -> np.ndarray:
    """Tag-square corners of a reference-style pose (no half-pixel shift), as the
    reference tests compare them (detector/tests/test_detector.cpp:51-60)."""
    return np.array([scenes.project(pose, x, y) for x, y in UNIT])


def corner_error(corners: np.ndarray, truth: np.ndarray) -> float:
    """Mean corner distance with corners matched as an unordered set
    (reference detector/bench/bench_detector.cpp:71-85)."""
    c = np.asarray(corners, dtype=np.float64).reshape(4, 2)
    t = np.asarray(truth, dtype=np.float64).reshape(4, 2)
    return min(float(np.mean([np.hypot(*(c[j] - t[p[j]])) for j in range(4)]))
               for p in itertools.permutations(range(4)))


def matches(corners: np.ndarray, truth: np.ndarray) -> bool:
    """Centre within 0.75 tag sides (reference bench_detector.cpp:52-65)."""
    c = np.asarray(corners, dtype=np.float64).reshape(4, 2)
    t = np.asarray(truth, dtype=np.float64).reshape(4, 2)
    side = np.mean([np.hypot(*(t[(j + 1) % 4] - t[j])) for j in range(4)])
    return bool(np.hypot(*(c.mean(0) - t.mean(0))) <= 0.75 * side)


def score(dets, count: int, truth_ids, truth_corners) -> tuple[int, int, int, list[float]]:
    """(tags, found, wrong ids, corner errors) for one frame."""
    found, errs = 0, []
    for tid, tc in zip(truth_ids, truth_corners):
        best = None
        for k in range(count):
            if dets["id"][k] != tid or not matches(dets["corners"][k], tc):
                continue
            e = corner_error(dets["corners"][k], tc)
            best = e if best is None else min(best, e)
        if best is not None:
            found += 1
            errs.append(best)
    wrong = sum(1 for k in range(count) if dets["id"][k] not in set(int(i) for i in truth_ids))
    return len(truth_ids), found, wrong, errs


def kat_multiple_frame():
    """The five-tag 1280x720 scene of the reference's test_multiple
    (detector/tests/test_detector.cpp:189-228)."""
    cases = [(3, (220, 180, 120, 0.2)), (17, (640, 180, 140, -0.35)), (101, (1050, 190, 110, 0.6)),
             (586, (420, 520, 150, 0.9)), (42, (950, 520, 100, -0.1))]
    img = np.full((720, 1280), 255, np.uint8)
    poses = {}
    for tid, (cx, cy, s, a) in cases:
        pose = scenes.make_pose(cx, cy, s, a)
        poses[tid] = pose
        img = np.minimum(img, scenes.render_tag(0, tid, 1280, 720, pose))
    return img, poses


def refit64_errors(frame, gray, quads32, hulls32, decodes):
    """Per decoded candidate: (max corner distance in px between the FP32
    quad and the oracle's FP64 re-fit, whether the FP64 hull quad is the same
    within 1e-3 px, relative max-abs difference of the result homography
    built from the FP32 corners and from the FP64 corners, in FP64)."""
    import oracle
    n = frame.candidate_count
    h64, q64 = frame.refit64(gray)
    q32 = np.asarray(quads32, dtype=np.float64)[:n * 8].reshape(n, 8)
    h32 = np.asarray(hulls32, dtype=np.float64)[:n * 8].reshape(n, 8)
    out = []
    for ci in range(n):
        if decodes["id"][ci] < 0 or np.isnan(q64[ci, 0]) or np.isnan(q32[ci, 0]):
            continue
        err = float(np.hypot(q32[ci, 0::2] - q64[ci, 0::2], q32[ci, 1::2] - q64[ci, 1::2]).max())
        same_hull = bool(np.abs(h32[ci] - h64[ci]).max() < 1e-3)
        rel = float("nan")
        c32 = decodes["corners"][ci].astype(np.float64)
        for r in range(4):  # the decoded rotation of the refined quad
            if np.array_equal(np.roll(q32[ci].reshape(4, 2), -r, axis=0).reshape(8), c32):
                hh64 = oracle.homography64(np.roll(q64[ci].reshape(4, 2), -r, axis=0).reshape(8))
                hh32 = oracle.homography64(c32)
                rel = float(np.abs(hh32 - hh64).max() / np.abs(hh64).max())
                break
        out.append((err, same_hull, rel))
    return out
