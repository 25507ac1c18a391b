"""Full-configuration parity sweeps of the CUDA pipeline against the CPU oracle
(gpu): every bd_config knob the reference honours, the whole 640x480 scene
set, all 600 1280x800 workload frames with both families, the reference
generator's full scene sets, and the first stage (tile extremes, histograms,
frame references) compared directly.

Final records are compared bit for bit on every frame; the per-stage dumps
(bitmap, runs, labels, area/bbox, candidates, hull and refined quads,
decodes) on every 16th frame, to keep the suite's run time small.
"""
import numpy as np
import pytest

import bdcudatag
import oracle
import scenes
from gpu_checks import check_frame, check_tile_stats, same_records
from helpers import score

pytestmark = pytest.mark.gpu


# --- every bd_config knob (gpu_detector.cu:1905-1943 resolves them) --------

KNOBS = [
    dict(refine_edges=0),                       # edge refinement off (:1200)
    dict(use_cuda_graph=0),                     # direct launches (:2051-2056, :2186-2194)
    dict(max_hamming=1),
    dict(max_hamming=2),
    dict(max_hamming=3),
    dict(max_hamming=9),                        # clamped to 3 (:1907-1909)
    dict(min_cluster_pixels=60),                # tag-like filter (:591-638)
    dict(min_cluster_pixels=0),                 # clamped to 1
    dict(min_tag_pixels=20),
    dict(min_tag_pixels=1),                     # clamped to 4
    dict(decode_sharpening=0.0),                # decode cells (:1376)
    dict(decode_sharpening=0.75),
    dict(min_decision_margin=0.0),
    dict(min_decision_margin=12.0),
    dict(max_candidates=16),                    # user cap at the clamp edges (:1918-1923)
    dict(max_candidates=1024),
    dict(max_candidates=5),                     # clamped to 16
    dict(max_candidates=100000),                # clamped to 1024
    dict(max_detections=1),
    dict(max_detections=256),
    dict(max_detections=1000),                  # clamped to 256
    dict(refine_edges=0, use_cuda_graph=0, max_hamming=0, decode_sharpening=0.5),
]


@pytest.mark.parametrize("knob", KNOBS, ids=[",".join(f"{k}={v}" for k, v in d.items()) for d in KNOBS])
def test_config_knobs(knob):
    frames = [scenes.render_scene(scenes.MIXED_1280, i, 1280, 800)[0] for i in (0, 5)]
    # The KAT frame with one flipped bit decodes at hamming 1 (or not at 0).
    pose = scenes.make_pose(320.0, 240.0, 170.0, 0.15)
    frames.append(scenes.render_tag(0, 0, 640, 480, pose, flip_one_bit=True))
    gcfg = bdcudatag.default_config(**knob)
    ocfg = oracle.default_config(**knob)
    for i, img in enumerate(frames):
        for fam in (0, 1):
            check_frame(img, fam, gcfg, ocfg, stages=(i == 0 or fam == 0))


# --- whole scene sets ----------------------------------------------------------

def test_config1_all_32_scenes():
    """The 32 seeded 640x480 scenes of eight tag36h11 tags each."""
    tags = found = wrong = 0
    for i in range(32):
        img, truth = scenes.render_scene(scenes.EIGHT_TAGS_640, i, 640, 480)
        n, d = check_frame(img, 0, stages=(i % 16 == 0))
        t, f, wr, _ = score(d, n, [t.id for t in truth if t.family == 0],
                            [t.corners for t in truth if t.family == 0])
        tags, found, wrong = tags + t, found + f, wrong + wr
    assert wrong == 0 and found >= 0.98 * tags


def test_config2_all_600_frames_both_families():
    """All 600 seeded 1280x800 workload frames, both families, as 4-camera
    batches (the benchmark's path) against the oracle run on every host
    thread; every 16th frame also through the single-frame path at every
    stage."""
    import os

    torch = pytest.importorskip("torch")
    count, cams = 600, 4
    frames, _ = scenes.render_many(scenes.MIXED_1280, [(1280, 800)] * count, threads=os.cpu_count() or 8)
    want, want_n = oracle.detect_many(frames, [3] * count, threads=os.cpu_count() or 8)
    batch = bdcudatag.Batch([(1280, 800, 3)] * cams)
    dev = torch.from_numpy(np.stack(frames)).cuda()
    for k in range(0, count, cams):
        found, out = batch.detect([dev[k + i] for i in range(cams)], [1280] * cams, device=True)
        for i in range(cams):
            for fam in (0, 1):
                n = int(want_n[k + i, fam])
                assert found[i, fam] == n, (k + i, fam)
                same_records(out[i, fam, :n], want[k + i, fam, :n])
    for i in range(0, count, 16):
        for fam in (0, 1):
            check_frame(frames[i], fam)


@pytest.mark.parametrize("w,h", [(640, 480), (1280, 720), (1280, 800), (1920, 1080)])
def test_reference_scenes_all_32(w, h):
    """The reference generator's full 32-scene sets (bench_detector.cpp's
    make_scenes, reproduced byte for byte): bit-exact against the oracle, and
    the reference's published recall and corner accuracy."""
    imgs, ids, corners = scenes.ref_scenes(w, h, 32)
    tags = found = wrong = 0
    errs = []
    for i in range(len(imgs)):
        n, d = check_frame(imgs[i], 0, bdcudatag.default_config(max_detections=32),
                           oracle.default_config(max_detections=32), stages=(i % 16 == 0))
        t, f, wr, e = score(d, n, ids[i], corners[i])
        tags, found, wrong, errs = tags + t, found + f, wrong + wr, errs + e
    assert found == tags and wrong == 0
    assert np.median(errs) < 0.3


# --- the first stage, directly ----------------------------------------------------

def _bright_noise(w, h, seed):
    rng = np.random.default_rng(seed)
    return rng.integers(236, 256, size=(h, w), dtype=np.uint8)


@pytest.mark.parametrize("stats_rows", [1, 2, 4])
def test_tile_stats_direct(stats_rows):
    """Tile min/max, the span and mean histograms and the frame references
    (noise-floor quartile, Otsu level) of k_stats against the oracle, for
    every rows-per-CTA shape, on frames of odd sizes and strides.

    4096x4096 bright noise puts the Otsu weighted sum just under 2^24 (the
    exact integer scan); 8192x2200 bright noise puts it above (the
    sequential FP32 loop of the reference)."""
    torch = pytest.importorskip("torch")
    cases = [scenes.render_scene(scenes.MIXED_1280, 3, 1280, 800)[0],
             scenes.render_scene(scenes.MULTI_SIZE, 2, 1001, 777)[0],
             scenes.render_scene(scenes.MULTI_SIZE, 4, 17, 23)[0],
             scenes.render_scene(scenes.MULTI_SIZE, 6, 2000, 40)[0],
             np.full((480, 640), 255, np.uint8),
             _bright_noise(4096, 4096, 1),
             _bright_noise(8192, 2200, 2)]
    for img in cases:
        h, w = img.shape
        ref = oracle.Frame(img, 0)
        s = int(np.dot(np.arange(64), ref.stage("mean_hist").astype(np.int64)))
        if (w, h) == (4096, 4096):
            assert s < (1 << 24)
        if (w, h) == (8192, 2200):
            assert s >= (1 << 24)
        for pad in (0, 3):  # 16-byte aligned rows, then unaligned rows
            batch = bdcudatag.Batch([(w, h, 1)])
            batch.set_launch(stats_rows=stats_rows)
            buf = torch.zeros((h, w + pad), dtype=torch.uint8, device="cuda")
            buf[:, :w] = torch.from_numpy(img).cuda()
            found, out = batch.detect([buf], [w + pad], device=True)
            check_tile_stats(batch.stage(0, "tile_min"), batch.stage(0, "tile_max"),
                             batch.stage(0, "state"), ref)
            n, want = ref.detections()
            assert found[0, 0] == n
            same_records(out[0, 0, :n], want)
