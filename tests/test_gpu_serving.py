"""Continuous-batching server (gpu): each frame's result in the mix equals
the result of detecting it alone with a single-frame detector, bit for bit
(tolerance 0: integer decodes, identical FP32 corners and homography)."""
import numpy as np
import pytest

import bdcudatag
import scenes

pytestmark = pytest.mark.gpu

CAMS = [(640, 480, 3), (1280, 800, 3), (1920, 1080, 1), (1600, 1304, 2), (3840, 2160, 3)]


def alone(frame, w, h, fams):
    out = {}
    for fam in (0, 1):
        if (fams >> fam) & 1:
            n, d = bdcudatag.Detector(fam, w, h).detect(frame)
            out[fam] = (n, d)
    return out


def test_results_same_alone_and_in_mix():
    torch = pytest.importorskip("torch")
    per_cam = 5
    frames = {}
    for c, (w, h, _) in enumerate(CAMS):
        imgs, _ = scenes.render_many(scenes.SERVING, [(w, h)] * per_cam, base=scenes.base_seed(scenes.SERVING) + 100 * c)
        pinned = torch.empty((per_cam, h, w), dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = np.stack(imgs)
        frames[c] = (imgs, pinned)
    server = bdcudatag.Server(CAMS, max_batches=3, queue_depth=per_cam)
    tickets = []
    for k in range(per_cam):
        for c in range(len(CAMS)):
            src = frames[c][1][k] if k % 2 == 0 else frames[c][0][k]  # pinned and pageable
            t = server.submit(c, src)
            assert t >= 0, bdcudatag.last_error()
            tickets.append((c, k, t))
    results = {}
    for c, k, t in tickets:
        rc, found, out, lat = server.wait(t)
        assert rc == 1 and lat > 0
        results[(c, k)] = (found, out)
    st = server.stats()
    assert st.completed == st.submitted == len(tickets)
    assert st.batches < len(tickets)  # frames were batched together
    assert 1 <= st.plans <= 3
    for (c, k), (found, out) in results.items():
        w, h, fams = CAMS[c]
        ref = alone(frames[c][0][k], w, h, fams)
        for fam in (0, 1):
            if fam not in ref:
                assert found[fam] == -1
                continue
            n, d = ref[fam]
            assert found[fam] == n
            assert out[fam, :n].tobytes() == d.tobytes()
    server.close()


def test_admission_and_rejection():
    w, h, fams = 640, 480, 1
    img, _ = scenes.render_scene(scenes.SERVING, 3, w, h)
    # A budget too small for one batch is refused at creation.
    with pytest.raises(RuntimeError):
        bdcudatag.Server([(w, h, fams)], device_budget=1 << 20)
    server = bdcudatag.Server([(w, h, fams)], max_batches=1, queue_depth=2)
    t0 = server.submit(0, img)
    t1 = server.submit(0, img)
    assert t0 >= 0 and t1 >= 0
    t2 = server.submit(0, img)  # third outstanding frame of this camera
    assert t2 == bdcudatag.ERROR_OUT_OF_MEMORY or t2 >= 0
    for t in (t0, t1) + ((t2,) if t2 >= 0 else ()):
        assert server.wait(t)[0] == 1
    if t2 < 0:
        assert server.stats().rejected == 1
    n, d = bdcudatag.Detector(0, w, h).detect(img)
    t3 = server.submit(0, img)
    rc, found, out, _ = server.wait(t3)
    assert found[0] == n and out[0, :n].tobytes() == d.tobytes()
    server.close()


def test_pressure_batches_and_refuses():
    """Submissions outpace completions: one batch plan in flight (a 3840x2160
    camera makes each launch long), every camera bursts six frames into a
    queue two deep.  The queue refuses the rest (admission), the waiting
    frames of several cameras share launches (continuous batching), and each
    admitted frame's result still equals detecting it alone."""
    torch = pytest.importorskip("torch")
    cams = [(3840, 2160, 3), (1280, 800, 3), (1280, 800, 1), (640, 480, 2)]
    burst, depth = 6, 2
    frames = {}
    for c, (w, h, _) in enumerate(cams):
        imgs, _ = scenes.render_many(scenes.SERVING, [(w, h)] * burst,
                                     base=scenes.base_seed(scenes.SERVING) + 700 + 50 * c)
        pinned = torch.empty((burst, h, w), dtype=torch.uint8, pin_memory=True)
        pinned.numpy()[:] = np.stack(imgs)
        frames[c] = (imgs, pinned)
    server = bdcudatag.Server(cams, max_batches=1, queue_depth=depth)
    accepted, refused = [], 0
    for k in range(burst):
        for c in range(len(cams)):
            t = server.submit(c, frames[c][1][k])
            if t >= 0:
                accepted.append((c, k, t))
            else:
                assert t == bdcudatag.ERROR_OUT_OF_MEMORY
                refused += 1
    assert refused == (burst - depth) * len(cams)
    results = {(c, k): server.wait(t) for c, k, t in accepted}
    st = server.stats()
    assert st.rejected == refused and st.completed == len(accepted) == depth * len(cams)
    assert st.mean_batch_frames > 1.0, st.mean_batch_frames
    for (c, k), (rc, found, out, _) in results.items():
        assert rc == 1
        w, h, fams = cams[c]
        ref = alone(frames[c][0][k], w, h, fams)
        for fam in (0, 1):
            if fam not in ref:
                assert found[fam] == -1
                continue
            n, d = ref[fam]
            assert found[fam] == n
            assert out[fam, :n].tobytes() == d.tobytes()
    server.close()
