"""C ABI checks that need no GPU: the library loads (no CPU fallback exists:
loading is the product path), exports every declared symbol with the
reference layouts, and rejects bad arguments before touching CUDA
(reference detector/tests/test_detector.cpp:342-370)."""
import ctypes
import re
import subprocess
from pathlib import Path

import bdcudatag

REPO = Path(__file__).resolve().parent.parent


def declared_symbols() -> set[str]:
    names = set()
    for h in (REPO / "include" / "bdcudatag").glob("*.h"):
        names |= set(re.findall(r"BD_API\s+[\w\s\*]+?\b(bd_\w+)\s*\(", h.read_text()))
    return names


def test_exports_every_declared_symbol():
    declared = declared_symbols()
    assert set(bdcudatag.REFERENCE_SYMBOLS) | set(bdcudatag.GB300_SYMBOLS) == declared
    out = subprocess.run(["nm", "-D", "--defined-only", str(bdcudatag.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (bd_\w+)$", out, re.M))
    assert declared <= exported, declared - exported
    lib = bdcudatag.lib()
    for name in declared:
        assert hasattr(lib, name)


def test_struct_layouts():
    assert ctypes.sizeof(bdcudatag.Config) == 40
    assert ctypes.sizeof(bdcudatag.Detection) == 84
    assert ctypes.sizeof(bdcudatag.Stats) == 40
    assert bdcudatag.Detection.homography.offset == 48
    assert bdcudatag.Detection.corners.offset == 12


def test_metadata_and_defaults():
    lib = bdcudatag.lib()
    assert lib.bd_api_version() == 2
    assert lib.bd_version_string() == b"bdcudatag 0.1.0"
    assert lib.bd_family_count() == 2
    assert lib.bd_family_name(0) == b"tag36h11" and lib.bd_family_name(1) == b"tag16h5"
    assert lib.bd_family_name(2) is None
    assert [lib.bd_family_bits_per_side(f) for f in (0, 1, 7)] == [6, 4, -1]
    assert [lib.bd_family_min_hamming(f) for f in (0, 1, -1)] == [11, 5, -1]
    assert [lib.bd_family_default_max_hamming(f) for f in (0, 1, 3)] == [2, 1, -1]
    c = bdcudatag.default_config()
    assert (c.struct_size, c.max_hamming, c.min_cluster_pixels, c.min_tag_pixels, c.max_detections,
            c.max_candidates, c.refine_edges, c.use_cuda_graph) == (40, -1, 24, 8, 64, 0, 1, 1)
    assert abs(c.min_decision_margin - 3.0) < 1e-7 and abs(c.decode_sharpening - 0.25) < 1e-7


def test_create_rejects_bad_arguments():
    lib = bdcudatag.lib()
    status = ctypes.c_int32(0)
    assert not lib.bd_detector_create(99, 640, 480, None, ctypes.byref(status))
    assert status.value == bdcudatag.ERROR_INVALID_ARGUMENT
    assert bdcudatag.last_error() == "unknown tag family"
    assert not lib.bd_detector_create(0, 0, 480, None, ctypes.byref(status))
    assert status.value == bdcudatag.ERROR_INVALID_ARGUMENT
    assert not lib.bd_detector_create(0, 8193, 480, None, ctypes.byref(status))
    small = bdcudatag.default_config(struct_size=8)
    assert not lib.bd_detector_create(0, 640, 480, ctypes.byref(small), ctypes.byref(status))
    assert "struct_size" in bdcudatag.last_error()
    cams = (bdcudatag.Camera * 1)(bdcudatag.Camera(640, 480, 4, 0))
    assert not lib.bd_batch_create(ctypes.cast(cams, ctypes.c_void_p), 1, None, ctypes.byref(status))
    assert status.value == bdcudatag.ERROR_INVALID_ARGUMENT
    assert lib.bd_detector_detect_host(None, None, 640, None, 0) == bdcudatag.ERROR_INVALID_ARGUMENT
    assert bdcudatag.last_error() == "null detector"
