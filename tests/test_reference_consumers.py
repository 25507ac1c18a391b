"""Drop-in checks with the reference's own consumers (CPU, only where the
reference checkout exists): its C++ known-answer test program and benchmark
compile unchanged against include/ and link to libbdcudatag.so with every
symbol resolved, and its Python ctypes backend
(detector/bench/compare_detectors.py:71-209) binds this library."""
import importlib.util
import os
import re
import subprocess
import sys
from pathlib import Path

import pytest

import bdcudatag

REPO = Path(__file__).resolve().parent.parent


def _reference_dir():
    """The reference checkout: BD_REFERENCE_DIR, else where oracle/build_ref.sh
    found it (recorded in oracle/_ref/REFERENCE_DIR), else None."""
    env = os.environ.get("BD_REFERENCE_DIR")
    if env:
        return Path(env)
    rec = REPO / "oracle" / "_ref" / "REFERENCE_DIR"
    return Path(rec.read_text().strip()) if rec.exists() else None


_ROOT = _reference_dir()
REF = _ROOT / "detector" if _ROOT else None
pytestmark = pytest.mark.skipif(REF is None or not REF.is_dir(), reason="reference checkout not present")


def test_reference_cpp_consumers_link():
    subprocess.run([str(REPO / "oracle" / "build_ref.sh")], check=True, capture_output=True)
    exported = set(re.findall(r" T (\S+)$", subprocess.run(
        ["nm", "-D", "--defined-only", str(bdcudatag.LIB_PATH)], capture_output=True, text=True,
        check=True).stdout, re.M))
    for prog in ("test_detector_on_gb300", "bench_detector_on_gb300"):
        binary = REPO / "oracle" / "_ref" / prog
        assert binary.exists()
        undefined = subprocess.run(["nm", "-D", "--undefined-only", str(binary)], capture_output=True,
                                   text=True, check=True).stdout
        wanted = set(re.findall(r" U (\S*(?:bd_|bdcudatag)\S*)$", undefined, re.M))
        assert wanted, prog
        assert wanted <= exported, wanted - exported
        ldd = subprocess.run(["ldd", str(binary)], capture_output=True, text=True).stdout
        assert "libbdcudatag.so" in ldd and "not found" not in ldd


def test_reference_ctypes_backend_binds():
    spec = importlib.util.spec_from_file_location("compare_detectors", REF / "bench" / "compare_detectors.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules["compare_detectors"] = mod
    spec.loader.exec_module(mod)
    backend = mod.BdcudatagBackend(str(bdcudatag.LIB_PATH), max_detections=32)
    assert backend.version == "bdcudatag 0.1.0"
    assert bdcudatag.ctypes.sizeof(backend._Detection) == 84
    backend.close()
