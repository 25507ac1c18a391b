"""The persistent launch (k_persistent.cu): one kernel per batch whose CTAs
pull (frame, stage, unit) items from a device work queue.  Its results must
equal the per-stage launches' and the oracle's bit for bit, for any grid
size and launch shape; a wait that runs out must end the batch with an error
status and leave the CUDA context usable (gpu)."""
import numpy as np
import pytest

import bdcudatag
import oracle
import scenes
from gpu_checks import check_tile_stats, same_records

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

SIZES = [(640, 480), (1280, 800), (1600, 1304), (1920, 1080)] * 4


def _mixed_batch():
    frames, _ = scenes.render_many(scenes.MULTI_SIZE, SIZES, threads=8,
                                   base=scenes.base_seed(scenes.MULTI_SIZE) + 900)
    frames[1] = scenes.render_scene(scenes.MIXED_1280, 5, 1280, 800)[0]  # candidates past the cap
    cams = [(w, h, (3, 1, 2, 3)[i % 4]) for i, (w, h) in enumerate(SIZES)]
    return frames, cams


def _check_against_oracle(found, out, frames, cams):
    for i, (w, h, fams) in enumerate(cams):
        for fam in (0, 1):
            if not (fams >> fam) & 1:
                assert found[i, fam] == -1
                continue
            n, want = oracle.Frame(frames[i], fam).detections()
            assert found[i, fam] == n, (i, fam)
            same_records(out[i, fam, :n], want)


@pytest.mark.parametrize("shape", [
    dict(persist_ctas=0),
    dict(persist_ctas=1),
    dict(persist_ctas=7, stats_rows=4, band_cap=256),
    dict(persist_ctas=152, quad_split=0),
    dict(persist_ctas=300, quad_split=16, band_cap=512, stats_rows=2),
], ids=lambda d: ",".join(f"{k}={v}" for k, v in d.items()))
def test_persistent_equals_staged_and_oracle(shape):
    frames, cams = _mixed_batch()
    dev = [torch.from_numpy(f).cuda() for f in frames]
    strides = [w for w, _ in SIZES]
    batch = bdcudatag.Batch(cams)
    found, out = batch.detect(dev, strides, device=True)
    batch.set_launch(persistent=1, **shape)
    for rep in range(2):  # the queue is cleared between batches
        f2, o2 = batch.detect(dev, strides, device=True)
        assert np.array_equal(f2, found) and o2.tobytes() == out.tobytes(), (shape, rep)
    # host input through the graph with the H2D copy
    f3, o3 = batch.detect(frames, strides)
    assert np.array_equal(f3, found) and o3.tobytes() == out.tobytes()
    # every stage of one frame
    ref = oracle.Frame(frames[5], 0)
    check_tile_stats(batch.stage(5, "tile_min"), batch.stage(5, "tile_max"), batch.stage(5, "state"), ref)
    rc = batch.stage(5, "row_count")
    assert np.array_equal(rc, ref.stage("row_count"))
    assert np.array_equal(batch.stage(5, "bits"), ref.stage("bits"))
    valid = (np.arange(ref.row_cap)[None, :] < rc[:, None]).ravel()
    lab = batch.stage(5, "label")[valid]
    assert np.array_equal(lab, ref.stage("label")[valid])
    nc = ref.candidate_count
    assert np.array_equal(batch.stage(5, "candidates")[:nc], ref.stage("candidates"))
    _check_against_oracle(found, out, frames, cams)


def test_persistent_direct_launch_and_workload_frames():
    """use_cuda_graph = 0 (direct launches) and 4-camera 1280x800 batches of
    the benchmark workload, both families."""
    frames, _ = scenes.render_many(scenes.MIXED_1280, [(1280, 800)] * 12, threads=8)
    cfg = bdcudatag.default_config(use_cuda_graph=0)
    batch = bdcudatag.Batch([(1280, 800, 3)] * 4, cfg)
    batch.set_launch(persistent=1)
    for k in range(0, 12, 4):
        found, out = batch.detect(frames[k:k + 4])
        _check_against_oracle(found, out, frames[k:k + 4], [(1280, 800, 3)] * 4)


def test_persistent_many_batches_in_flight():
    """Batches on several streams at once (the benchmark's pipelined loop),
    then the last batch's results against the oracle."""
    frames, _ = scenes.render_many(scenes.MIXED_1280, [(1280, 800)] * 8, threads=8)
    dev = torch.from_numpy(np.stack(frames)).cuda()
    sets = [[dev[(k * 4 + i) % 8] for i in range(4)] for k in range(2)]
    batches = [bdcudatag.Batch([(1280, 800, 3)] * 4) for _ in range(6)]
    streams = [torch.cuda.Stream() for _ in batches]
    for b, s in zip(batches, streams):
        b.set_launch(persistent=1, persist_ctas=64)
        b.set_stream(s)
    wall, lat = bdcudatag.pipeline(batches, sets, [1280] * 4, 60, True)
    assert len(lat) == 60
    # batch j ran steps j, j + 6, ...; step 54 + j used set (54 + j) % 2
    for j, b in enumerate(batches):
        found, out = b.wait()
        k = (54 + j) % 2
        _check_against_oracle(found, out, frames[4 * k:4 * k + 4], [(1280, 800, 3)] * 4)


def test_persistent_wait_runs_out_and_context_survives():
    """A withheld work item (the test hook: nothing ever publishes it) makes a
    CTA's bounded queue wait run out: the batch ends with an error status,
    every CTA leaves, and the next batch on the same context is correct."""
    frames, _ = scenes.render_many(scenes.MIXED_1280, [(1280, 800)] * 2, threads=8)
    batch = bdcudatag.Batch([(1280, 800, 3)] * 2)
    batch.set_launch(persistent=1, persist_ctas=16)
    batch.debug_persist(timeout_ns=50_000_000, stall_frame=1)
    with pytest.raises(RuntimeError, match="timed out"):
        batch.detect(frames)
    batch.debug_persist(timeout_ns=1_000_000_000, stall_frame=-1)
    found, out = batch.detect(frames)
    _check_against_oracle(found, out, frames, [(1280, 800, 3)] * 2)
    torch.cuda.synchronize()
    # an unrelated CUDA operation on the same context still works
    assert float(torch.ones(4, device="cuda").sum()) == 4.0
