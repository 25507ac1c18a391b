"""CUDA pipeline versus the CPU oracle, through the C ABI (gpu).

Bit-exact: the bitmap, runs, component labels, area/bbox at roots, the
candidate list, hull and refined quads, per-candidate decodes and the final
records (id, hamming, margin, corners, homography).  The oracle is pinned to
the reference in test_oracle_pin.py.
"""
import numpy as np
import pytest

import bdcudatag
import oracle
import scenes
from gpu_checks import check_frame, kat_config, okat_config, same_records
from helpers import kat_multiple_frame, pose_corners, score

pytestmark = pytest.mark.gpu
W, H = 640, 480


# --- the reference's own known-answer tests (test_detector.cpp) -------------

@pytest.mark.parametrize("family,tag_id,size", [(0, 0, 170), (1, 0, 120)])
def test_centered_tag(family, tag_id, size):
    pose = scenes.make_pose(W * 0.5, H * 0.5, size, 0.0)
    n, d = check_frame(scenes.render_tag(family, tag_id, W, H, pose), family, kat_config(), okat_config())
    assert n == 1 and d["id"][0] == tag_id and d["hamming"][0] == 0 and d["decision_margin"][0] > 2.0
    assert np.abs(d["corners"][0].reshape(4, 2) - pose_corners(pose)).max() <= 2.5


def test_rotations_hamming_small_homography():
    for r in range(4):
        pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, r * 1.5707963267948966)
        n, d = check_frame(scenes.render_tag(0, 0, W, H, pose), 0, kat_config(), okat_config())
        assert n == 1 and d["id"][0] == 0
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, 0.15)
    img = scenes.render_tag(0, 0, W, H, pose, flip_one_bit=True)
    n, d = check_frame(img, 0, kat_config(), okat_config())
    assert n == 1 and d["hamming"][0] == 1
    n, _ = check_frame(img, 0, kat_config(max_hamming=0), okat_config(max_hamming=0))
    assert n == 0
    pose = scenes.make_pose(W * 0.5, H * 0.5, 38.0, 0.25)
    n, d = check_frame(scenes.render_tag(0, 7, W, H, pose), 0, kat_config(), okat_config())
    assert n == 1 and d["id"][0] == 7
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, 0.3, 0.00035)
    n, d = check_frame(scenes.render_tag(0, 5, W, H, pose), 0, kat_config(), okat_config())
    Hm = d["homography"][0].astype(np.float64)
    assert abs(Hm[8] - 1.0) <= 1e-5
    c = d["corners"][0].reshape(4, 2)
    for i, (tx, ty) in enumerate([(-1, -1), (1, -1), (1, 1), (-1, 1)]):
        w = Hm[6] * tx + Hm[7] * ty + Hm[8]
        assert abs((Hm[0] * tx + Hm[1] * ty + Hm[2]) / w - c[i, 0]) <= 0.01


def test_multiple_and_blank():
    img, poses = kat_multiple_frame()
    n, d = check_frame(img, 0, kat_config(), okat_config())
    assert n == 5 and sorted(d["id"]) == sorted(poses)
    det = bdcudatag.Detector(0, W, H, kat_config())
    for v in (255, 0):
        n, _ = det.detect(np.full((H, W), v, np.uint8))
        assert n == 0
    assert det.stats().roi_rows == 0


def test_device_path_and_stride():
    torch = pytest.importorskip("torch")
    pose = scenes.make_pose(W * 0.5, H * 0.5, 150.0, 0.1)
    img = scenes.render_tag(0, 11, W, H, pose)
    det = bdcudatag.Detector(0, W, H, kat_config())
    n_host, host = det.detect(img)
    padded = np.full((H, W + 96), 7, np.uint8)
    padded[:, :W] = img
    t = torch.from_numpy(padded).cuda()
    n, dev = det.detect_device(t, W + 96)
    assert n == n_host == 1 and dev["id"][0] == 11
    same_records(dev, host)
    n2, strided = det.detect(padded[:, :W], stride=W + 96)
    same_records(strided, host)


def test_thread_safety():
    import threading
    pose = scenes.make_pose(W * 0.5, H * 0.5, 170.0, 0.0)
    img = scenes.render_tag(0, 0, W, H, pose)
    det = bdcudatag.Detector(0, W, H, kat_config())
    bad = []

    def work():
        local = bdcudatag.Detection()
        for _ in range(5):
            n = bdcudatag.lib().bd_detector_detect_host(det.handle, img.ctypes.data, W,
                                                        bdcudatag.ctypes.addressof(local), 1)
            if n != 1 or local.id != 0:
                bad.append(n)

    threads = [threading.Thread(target=work) for _ in range(4)]
    [t.start() for t in threads]
    [t.join() for t in threads]
    assert not bad and det.stats().frames == 20


# --- workload frames and edge cases -------------------------------------------

@pytest.mark.parametrize("index", range(8))
def test_mixed_1280_frames_both_families(index):
    img, truth = scenes.render_scene(scenes.MIXED_1280, index, 1280, 800)
    for fam in (0, 1):
        check_frame(img, fam, stages=(index % 4 == 0 or index == 5))


@pytest.mark.parametrize("w,h", [(16, 16), (17, 23), (1001, 777), (33, 300), (2000, 40)])
def test_odd_sizes(w, h):
    img, _ = scenes.render_scene(scenes.MULTI_SIZE, w * 7 + h, w, h)
    check_frame(img, 0)
    check_frame(np.ascontiguousarray(img[::-1]), 1)


def test_dense_bands_4k():
    # 3840x2160 serving frames hold 8-row bands of up to ~5000 runs: more
    # than one shared-memory segment (default cap 2048), so those bands are
    # labelled in row segments joined by k_merge.
    img, _ = scenes.render_scene(scenes.SERVING, 0, 3840, 2160)
    h, w = img.shape
    rc = oracle.Frame(img, 0).stage("row_count").astype(np.int64)
    pad = np.zeros(((h + 7) // 8) * 8, np.int64)
    pad[:h] = rc[:h]
    assert pad.reshape(-1, 8).sum(1).max() > 2048  # the segmented path is exercised
    for fam in (0, 1):
        check_frame(img, fam, stages=(fam == 0))


def test_single_row_over_cap_fallback():
    # Pixel noise at 8192 px width: rows of ~2000+ runs.  With band_cap 512
    # one row alone exceeds the cap, so the band takes the one-root-per-run
    # fallback; results equal the default shapes and the oracle.
    rng = np.random.default_rng(77)
    img = rng.integers(0, 256, size=(96, 8192), dtype=np.uint8)
    img[20:70, 1000:1060] = 30  # a dark block so some components are large
    n0, ref = check_frame(img, 0)
    torch = pytest.importorskip("torch")
    batch = bdcudatag.Batch([(8192, 96, 1)])
    batch.set_launch(band_cap=512)
    found, out = batch.detect([torch.from_numpy(img).cuda()], [8192], device=True)
    assert found[0, 0] == n0 and out[0, 0, :n0].tobytes() == ref.tobytes()
    lab_fb = batch.stage(0, "label")
    batch.set_launch(band_cap=2048)
    batch.detect([torch.from_numpy(img).cuda()], [8192], device=True)
    rc = batch.stage(0, "row_count")
    valid = (np.arange(8192 // 2 + 2)[None, :] < rc[:, None]).ravel()
    assert np.array_equal(lab_fb[valid], batch.stage(0, "label")[valid])


def test_caps_exceeded():
    # Clutter frame (index 5) pushes candidates past a small cap; a tiny
    # detection cap truncates in candidate order.
    img, _ = scenes.render_scene(scenes.MIXED_1280, 5, 1280, 800)
    check_frame(img, 0, bdcudatag.default_config(max_candidates=16, max_detections=2),
                oracle.default_config(max_candidates=16, max_detections=2))
    det = bdcudatag.Detector(0, 1280, 800, bdcudatag.default_config(max_detections=4))
    n, d = det.detect(img, capacity=0)
    assert len(d) == 0 and n == oracle.Frame(img, 0, oracle.default_config(max_detections=4)).detections()[0]


def test_batch_matches_single_frames():
    sizes = [(640, 480), (1280, 800), (1600, 1304), (1920, 1080)] * 2
    frames, _ = scenes.render_many(scenes.MULTI_SIZE, sizes, threads=8)
    cams = [(w, h, (3, 1, 2)[i % 3]) for i, (w, h) in enumerate(sizes)]  # both, 36h11, 16h5
    batch = bdcudatag.Batch(cams)
    found, out = batch.detect(frames)
    for i, (w, h, fams) in enumerate(cams):
        for fam in (0, 1):
            if not (fams >> fam) & 1:
                assert found[i, fam] == -1
                continue
            wn, want = oracle.Frame(frames[i], fam).detections()
            assert found[i, fam] == wn
            same_records(out[i, fam, :wn], want)
    # device input, second call on the same plan
    torch = pytest.importorskip("torch")
    dev = [torch.from_numpy(f).cuda() for f in frames]
    found2, out2 = batch.detect(dev, strides=[w for w, _ in sizes], device=True)
    assert np.array_equal(found2, found)
    for i in range(len(cams)):
        for fam in (0, 1):
            if found[i, fam] > 0:
                same_records(out2[i, fam, :found[i, fam]], out[i, fam, :found[i, fam]])


def test_batch_pinned_stream_query_profile():
    torch = pytest.importorskip("torch")
    sizes = [(1280, 800)] * 4
    frames, _ = scenes.render_many(scenes.MIXED_1280, sizes, threads=8)
    pinned = torch.empty((4, 800, 1280), dtype=torch.uint8, pin_memory=True)
    pinned.numpy()[:] = np.stack(frames)
    batch = bdcudatag.Batch([(1280, 800, 3)] * 4)
    found, out = batch.detect(frames)  # pageable: staged copy
    f2, o2 = batch.detect([pinned[i] for i in range(4)], strides=[1280] * 4)  # pinned: direct DMA
    assert np.array_equal(found, f2) and np.array_equal(out.view(np.uint8), o2.view(np.uint8))
    stream = torch.cuda.Stream()
    batch.set_stream(stream)
    batch.submit([pinned[i] for i in range(4)], strides=[1280] * 4)
    stream.synchronize()
    assert batch.query()
    f3, o3 = batch.wait()
    assert np.array_equal(found, f3) and np.array_equal(out.view(np.uint8), o3.view(np.uint8))
    batch.set_stream(None)
    dev = [torch.from_numpy(f).cuda() for f in frames]
    prof = batch.profile_device(dev, [1280] * 4)
    assert len(prof) == 8 and all(v >= 0 for v in prof.values())
    f4, o4 = batch.wait()
    assert np.array_equal(found, f4)
    for i in range(4):
        for fam in (0, 1):
            n, want = oracle.Frame(frames[i], fam).detections()
            assert found[i, fam] == n
            same_records(out[i, fam, :n], want)


def test_launch_shapes_and_autotune_keep_results():
    torch = pytest.importorskip("torch")
    sizes = [(640, 480), (1280, 800), (1600, 1304), (1920, 1080)] * 4
    frames, _ = scenes.render_many(scenes.MULTI_SIZE, sizes, threads=8, base=scenes.base_seed(scenes.MULTI_SIZE) + 500)
    dev = [torch.from_numpy(f).cuda() for f in frames]
    strides = [w for w, _ in sizes]
    batch = bdcudatag.Batch([(w, h, 3) for w, h in sizes])
    found, out = batch.detect(dev, strides, device=True)
    shapes = [dict(stats_rows=2, band_cap=256), dict(stats_rows=4, quad_warps=2, quad_split=0),
              dict(quad_ctas_per_sm=1, quad_warps=2, quad_split=16, band_cap=512),
              dict(stats_rows=1, quad_warps=8, quad_ctas_per_sm=16, quad_split=96, band_cap=2048),
              dict(fit_merged=1), dict(fit_merged=1, quad_split=0),
              dict(fit_merged=1, quad_split=16, band_cap=512)]
    for shape in shapes:
        batch.set_launch(**shape)
        f2, o2 = batch.detect(dev, strides, device=True)
        assert np.array_equal(f2, found) and o2.tobytes() == out.tobytes(), shape
    best, ms = batch.autotune(dev, strides, iterations=4)
    assert ms > 0 and best["quad_warps"] in (2, 4, 8)
    f3, o3 = batch.detect(dev, strides, device=True)
    assert np.array_equal(f3, found) and o3.tobytes() == out.tobytes()
    with pytest.raises(RuntimeError):
        batch.set_launch(stats_rows=3)
    with pytest.raises(RuntimeError):
        batch.set_launch(quad_warps=3)
    # the single-frame path agrees with the batch
    for i in (0, 5, 10, 15):
        w, h = sizes[i]
        for fam in (0, 1):
            n, d = bdcudatag.Detector(fam, w, h).detect(frames[i])
            assert found[i, fam] == n and out[i, fam, :n].tobytes() == d.tobytes()


def test_pipeline_runner_checks_and_results():
    torch = pytest.importorskip("torch")
    img, _ = scenes.render_scene(scenes.MIXED_1280, 2, 1280, 800)
    frame = torch.from_numpy(img).cuda()
    a = bdcudatag.Batch([(1280, 800, 3)])
    b = bdcudatag.Batch([(1280, 800, 3)])
    other = bdcudatag.Batch([(640, 480, 3)])
    with pytest.raises(RuntimeError):
        bdcudatag.pipeline([a, other], [[frame]], [1280], 2, True)  # different cameras
    with pytest.raises(RuntimeError):
        bdcudatag.pipeline([a, a], [[frame]], [1280], 2, True)  # the same batch twice
    with pytest.raises(RuntimeError):
        bdcudatag.pipeline([a, b], [[frame]], [1000], 2, True)  # stride below the width
    wall, lat = bdcudatag.pipeline([a, b], [[frame]], [1280], 5, True)
    assert wall > 0 and len(lat) == 5 and all(v > 0 for v in lat)
    found, out = b.wait()  # the last batch on b holds the frame's results
    for fam in (0, 1):
        n, want = oracle.Frame(img, fam).detections()
        assert found[0, fam] == n
        same_records(out[0, fam, :n], want)


def test_gpu_corners_against_fp64_refit():
    """The GPU's FP32 quads against the oracle's FP64 re-fit of the same
    candidates (hull, quad and edge refinement in double precision): the
    error statement of test_refit64.py, made on the CUDA results."""
    from helpers import refit64_errors
    rows = []
    for i in range(8):
        img, _ = scenes.render_scene(scenes.MIXED_1280, i, 1280, 800)
        for fam in (0, 1):
            det = bdcudatag.Detector(fam, 1280, 800)
            det.detect(img)
            ref = oracle.Frame(img, fam)
            nc = ref.candidate_count
            q = det.stage("quads")[fam * ref.max_candidates * 8:][:nc * 8]
            hq = det.stage("hull_quads")[:nc * 8]
            dg = det.stage("decodes")[fam * ref.max_candidates:][:nc]
            rows += refit64_errors(ref, img, q, hq, dg)
    assert len(rows) >= 50
    err = np.array([r[0] for r in rows])
    same = np.array([r[1] for r in rows])
    rel = np.array([r[2] for r in rows])
    assert same.mean() >= 0.85
    assert np.median(err[same]) < 5e-3 and err[same].max() < 0.1
    assert np.mean(err > 0.1) <= 0.05
    assert np.nanmedian(rel[same]) < 1e-4


@pytest.mark.parametrize("merged", [0, 1])
@pytest.mark.parametrize("split", [0, 32, 48, 96])
def test_fit_work_lists_split_candidates_by_size(split, merged):
    """k_cand_count's placing CTA lists the candidates above the split (for
    the CTA path) and the rest (for the warp path); every candidate is on
    exactly one list, and the results do not depend on the split."""
    torch = pytest.importorskip("torch")
    sizes = [(1280, 800), (640, 480), (1920, 1080)]
    frames = [scenes.render_scene(scenes.MIXED_1280, 5, 1280, 800)[0],
              scenes.render_scene(scenes.EIGHT_TAGS_640, 3, 640, 480)[0],
              scenes.render_scene(scenes.MULTI_SIZE, 9, 1920, 1080)[0]]
    batch = bdcudatag.Batch([(w, h, 3) for w, h in sizes])
    batch.set_launch(quad_split=split, fit_merged=merged)
    found, out = batch.detect([torch.from_numpy(f).cuda() for f in frames], [w for w, _ in sizes],
                              device=True)
    for i, img in enumerate(frames):
        ref = oracle.Frame(img, 0)
        nc = min(ref.candidate_count, ref.max_candidates)
        state = batch.stage(i, "state")
        # FrameState: counts[5], top_enc, bottom_enc, ref[2], done_stats,
        # done_cands, n_candidates, n_big, n_small, ...
        n_candidates, n_big, n_small = int(state[11]), int(state[12]), int(state[13])
        assert n_candidates == nc and n_big + n_small == nc
        bb = ref.stage("bbox").reshape(-1, 4)[ref.stage("candidates")[:nc]].astype(np.int64)
        side = np.maximum(bb[:, 2] - bb[:, 0], bb[:, 3] - bb[:, 1]) + 1
        assert n_big == (int(np.sum(side > split)) if split > 0 else 0)
        for fam in (0, 1):
            wn, want = oracle.Frame(img, fam).detections()
            assert found[i, fam] == wn
            same_records(out[i, fam, :wn], want)


def _ccl_patterns():
    """Binary-ish frames that stress connected-component labelling: a comb
    (many bars joined only at the top), a zigzag snake crossing every band,
    a checkerboard (8-connected diagonal joins only), and noise of several
    densities."""
    h, w = 240, 512
    comb = np.full((h, w), 220, np.uint8)
    comb[20:200, 40:480:6] = 30
    comb[20:24, 40:480] = 30
    snake = np.full((h, w), 220, np.uint8)
    for k, y in enumerate(range(10, 230, 6)):
        snake[y:y + 3, 20:490] = 30
        x = 487 if k % 2 == 0 else 20
        snake[y:y + 9, x:x + 3] = 30
    board = np.full((h, w), 220, np.uint8)
    yy, xx = np.mgrid[0:h, 0:w]
    board[((yy // 2) + (xx // 2)) % 2 == 0] = 30
    board[:8], board[-8:], board[:, :8], board[:, -8:] = 220, 220, 220, 220
    rng = np.random.default_rng(5)
    noise = [np.where(rng.random((h, w)) < p, 30, 220).astype(np.uint8) for p in (0.3, 0.5, 0.6)]
    return [comb, snake, board] + noise


@pytest.mark.parametrize("band_cap", [256, 2048])
def test_ccl_stress_patterns(band_cap):
    """Labels, areas and boxes bit-exact on adversarial component shapes,
    with small (many row segments) and large shared-memory band caps."""
    torch = pytest.importorskip("torch")
    frames = _ccl_patterns()
    h, w = frames[0].shape
    batch = bdcudatag.Batch([(w, h, 1)] * len(frames))
    batch.set_launch(band_cap=band_cap)
    found, out = batch.detect([torch.from_numpy(f).cuda() for f in frames], [w] * len(frames),
                              device=True)
    for i, img in enumerate(frames):
        ref = oracle.Frame(img, 0)
        rc = batch.stage(i, "row_count")
        assert np.array_equal(rc, ref.stage("row_count"))
        valid = (np.arange(ref.row_cap)[None, :] < rc[:, None]).ravel()
        lab = batch.stage(i, "label")[valid]
        assert np.array_equal(lab, ref.stage("label")[valid])
        roots = np.unique(lab)
        assert np.array_equal(batch.stage(i, "area")[roots], ref.stage("area")[roots])
        assert np.array_equal(batch.stage(i, "bbox").reshape(-1, 4)[roots],
                              ref.stage("bbox").reshape(-1, 4)[roots])
        wn, want = ref.detections()
        assert found[i, 0] == wn
        same_records(out[i, 0, :wn], want)
