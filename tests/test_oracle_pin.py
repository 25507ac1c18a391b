"""Pins the CPU oracle to the reference: its known-answer tests
(detector/tests/test_detector.cpp) and its benchmark scenes with published
accuracy (README.md:140-155), on CPU.  The oracle is the checker the CUDA
pipeline is compared against in the gpu tests."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
import scenes
from helpers import kat_multiple_frame, pose_corners, score

W, H = 640, 480
GOLDEN = Path(__file__).resolve().parent / "golden" / "ref_scenes.json"


def kat_config(**kw):
    # test_config() of the reference tests (test_detector.cpp:39-44)
    return oracle.default_config(max_detections=32, min_decision_margin=2.0, **kw)


def detect(img, family=0, cfg=None):
    f = oracle.Frame(img, family, cfg or kat_config())
    n, d = f.detections(32)
    return n, d, f


@pytest.mark.parametrize("family,tag_id,size", [(0, 0, 170), (1, 0, 120)])
def test_centered_tag(family, tag_id, size):
    pose = scenes.make_pose(W * 0.5, H * 0.5, size, 0.0)
    n, d, f = detect(scenes.render_tag(family, tag_id, W, H, pose), family)
    assert n == 1
    assert d["id"][0] == tag_id and d["hamming"][0] == 0 and d["decision_margin"][0] > 2.0
    assert np.abs(d["corners"][0].reshape(4, 2) - pose_corners(pose)).max() <= 2.5
    assert f.counts()[0] >= 1


@pytest.mark.parametrize("r", range(4))
def test_rotations(r):
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, r * 1.5707963267948966)
    n, d, _ = detect(scenes.render_tag(0, 0, W, H, pose))
    assert n == 1 and d["id"][0] == 0
    assert np.abs(d["corners"][0].reshape(4, 2) - pose_corners(pose)).max() <= 2.5


def test_hamming():
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, 0.15)
    img = scenes.render_tag(0, 0, W, H, pose, flip_one_bit=True)
    n, d, _ = detect(img)
    assert n == 1 and d["id"][0] == 0 and d["hamming"][0] == 1
    n, _, _ = detect(img, cfg=kat_config(max_hamming=0))
    assert n == 0


def test_multiple():
    img, poses = kat_multiple_frame()
    n, d, _ = detect(img)
    assert n == 5 and sorted(d["id"][:n]) == sorted(poses)
    for k in range(n):
        assert np.abs(d["corners"][k].reshape(4, 2) - pose_corners(poses[int(d["id"][k])])).max() <= 3.0


def test_small_tag():
    pose = scenes.make_pose(W * 0.5, H * 0.5, 38.0, 0.25)
    n, d, _ = detect(scenes.render_tag(0, 7, W, H, pose))
    assert n == 1 and d["id"][0] == 7
    assert np.abs(d["corners"][0].reshape(4, 2) - pose_corners(pose)).max() <= 4.0


def test_blank():
    for value in (255, 0):
        n, _, f = detect(np.full((H, W), value, np.uint8))
        assert n == 0
    # roiRows == 0 on a blank frame (java-api BDTagDetectorTest.java:59-70)
    assert f.counts()[4] == 0


def test_homography():
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, 0.3, 0.00035)
    n, d, _ = detect(scenes.render_tag(0, 5, W, H, pose))
    assert n == 1
    Hm = d["homography"][0].astype(np.float64)
    c = d["corners"][0].reshape(4, 2)
    for i, (tx, ty) in enumerate([(-1, -1), (1, -1), (1, 1), (-1, 1)]):
        w = Hm[6] * tx + Hm[7] * ty + Hm[8]
        assert abs((Hm[0] * tx + Hm[1] * ty + Hm[2]) / w - c[i, 0]) <= 0.01
        assert abs((Hm[3] * tx + Hm[4] * ty + Hm[5]) / w - c[i, 1]) <= 0.01
    assert abs(Hm[8] - 1.0) <= 1e-5
    gx, gy = scenes.project(pose, 0.0, 0.0)
    assert abs(Hm[2] / Hm[8] - gx) <= 3.0 and abs(Hm[5] / Hm[8] - gy) <= 3.0


# Published bdcudatag accuracy on these scenes (README.md:140-155):
# recall 100%, 0 wrong ids, median corner error (px).
PUBLISHED = {"640x480": 0.13, "1280x720": 0.17, "1280x800": 0.17, "1920x1080": 0.23}


@pytest.mark.parametrize("key", sorted(PUBLISHED))
def test_reference_scenes(key):
    fx = json.loads(GOLDEN.read_text())["resolutions"][key]
    w, h = map(int, key.split("x"))
    count = 8
    imgs, ids, corners = scenes.ref_scenes(w, h, count)
    errs, tags, found, wrong = [], 0, 0, 0
    for i in range(count):
        # The renderer reproduces the reference exporter's frame exactly.
        assert hashlib.sha256(imgs[i].tobytes()).hexdigest() == fx[i]["sha256"]
        truth = np.array([t["corners"] for t in fx[i]["tags"]])
        assert np.abs(truth - corners[i]).max() < 6e-4
        n, d = oracle.Frame(imgs[i], 0, oracle.default_config(max_detections=32)).detections(32)
        t, fnd, wr, e = score(d, n, ids[i], corners[i])
        tags, found, wrong, errs = tags + t, found + fnd, wrong + wr, errs + e
    assert found == tags and wrong == 0
    assert abs(float(np.median(errs)) - PUBLISHED[key]) < 0.03
