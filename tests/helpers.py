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
