"""bd_tile_stats_device_noalloc: the allocation-free entry point (gpu).

It exists for callers that may not allocate memory while they run (camera
callbacks, fixed-memory real-time systems, plugins inside another
framework's allocator).  This file is collected last so that a failure here
comes after every other test has run.  Its output must equal what the
existing detector entry point computes for the same frame: the tile min/max
of bd_detector_detect_device's first stage and the frame references in its
state record (tile values are integers: tolerance 0).  Two calls in a row
check that the shared scratch array is cleared between calls.
"""
import ctypes

import numpy as np
import pytest

import bdcudatag
import scenes

pytestmark = pytest.mark.gpu


def reference_stats(img, stride_img):
    """Tile min/max and frame references from the existing detector path."""
    h, w = img.shape
    det = bdcudatag.Detector(0, w, h)
    det.detect_device(stride_img, stride_img.stride(0))
    state = det.stage("state")
    # FrameState: counts[5], top_enc, bottom_enc, ref[2], ...
    return det.stage("tile_min"), det.stage("tile_max"), (int(state[7]), int(state[8]), int(state[4]))


def test_noalloc_matches_detector_twice():
    torch = pytest.importorskip("torch")
    lib = bdcudatag.lib()
    frames = [scenes.render_scene(scenes.MIXED_1280, 5, 1280, 800)[0], scenes.render_scene(scenes.MULTI_SIZE, 11, 1001, 777)[0]]
    stream = torch.cuda.current_stream()
    for img in frames:  # two calls in a row, different sizes and contents
        h, w = img.shape
        padded = torch.zeros((h, w + 64), dtype=torch.uint8, device="cuda")
        padded[:, :w] = torch.from_numpy(img).cuda()
        gray = padded[:, :w]
        t = ((w + 7) // 8) * ((h + 7) // 8)
        tmin = torch.full((t,), 7, dtype=torch.uint8, device="cuda")
        tmax = torch.full((t,), 7, dtype=torch.uint8, device="cuda")
        frame = torch.full((3,), 12345, dtype=torch.int32, device="cuda")
        rc = lib.bd_tile_stats_device_noalloc(gray.data_ptr(), w, h, w + 64, tmin.data_ptr(),
                                              tmax.data_ptr(), frame.data_ptr(),
                                              ctypes.c_void_p(stream.cuda_stream))
        assert rc == bdcudatag.OK, bdcudatag.last_error()
        torch.cuda.synchronize()
        want_min, want_max, want_frame = reference_stats(img, gray)
        assert np.array_equal(tmin.cpu().numpy(), want_min)
        assert np.array_equal(tmax.cpu().numpy(), want_max)
        assert tuple(int(v) for v in frame.cpu().numpy()) == want_frame


def test_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    lib = bdcudatag.lib()
    buf = torch.zeros(64, dtype=torch.uint8, device="cuda")
    p = buf.data_ptr()
    assert lib.bd_tile_stats_device_noalloc(p, 8193, 16, 8193, p, p, p, None) == \
        bdcudatag.ERROR_INVALID_ARGUMENT
    assert "out of range" in bdcudatag.last_error()
    assert lib.bd_tile_stats_device_noalloc(p, 16, 16, 8, p, p, p, None) == \
        bdcudatag.ERROR_INVALID_ARGUMENT
    assert lib.bd_tile_stats_device_noalloc(None, 16, 16, 16, p, p, p, None) == \
        bdcudatag.ERROR_INVALID_ARGUMENT
