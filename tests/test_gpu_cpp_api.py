"""The C++ API (bdcudatag::Detector, include/bdcudatag/detector.hpp) on the
GPU: a C++ program of this project, written against the public headers as a
reference caller would (tests/cpp/detector_api_check.cpp), compiled with g++
and linked to libbdcudatag.so, detects from host and device memory, moves the
detector and provokes the API's exceptions; its detections must equal the
CPU oracle's bit for bit (gpu)."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import bdcudatag
import oracle
import scenes

pytestmark = pytest.mark.gpu
REPO = Path(__file__).resolve().parent.parent


def _build(tmp_path):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    exe = tmp_path / "detector_api_check"
    lib_dir = Path(bdcudatag.LIB_PATH).parent
    subprocess.run(["g++", "-O1", "-std=c++17", f"-I{REPO / 'include'}", "-I/usr/local/cuda/include",
                    str(REPO / "tests" / "cpp" / "detector_api_check.cpp"), "-o", str(exe),
                    f"-L{lib_dir}", "-lbdcudatag", "-L/usr/local/cuda/lib64", "-lcudart",
                    f"-Wl,-rpath,{lib_dir}"], check=True)
    return exe


def _hex(v):
    return int(np.float32(v).view(np.uint32))


@pytest.mark.parametrize("family", [0, 1])
def test_cpp_detector_api(tmp_path, family):
    exe = _build(tmp_path)
    img, _ = scenes.render_scene(scenes.MIXED_1280, 2, 1280, 800)
    frame = tmp_path / "frame.raw"
    with open(frame, "wb") as fh:
        fh.write(b"1280 800\n")
        fh.write(img.tobytes())
    out = subprocess.run([str(exe), str(frame), str(family)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.splitlines()
    for name in ("capacity", "device", "move", "exceptions", "stats"):
        assert f"check {name} ok" in lines
    got = [ln.split()[1:] for ln in lines if ln.startswith("det ")]
    n, want = oracle.Frame(img, family).detections()
    assert len(got) == n and n > 0
    for row, d in zip(got, want):
        assert int(row[0]) == d["id"] and int(row[1]) == d["hamming"]
        vals = [int(x, 16) for x in row[2:]]
        ref = [_hex(d["decision_margin"])] + [_hex(c) for c in d["corners"]] + \
              [_hex(v) for v in d["homography"]]
        assert vals == ref
