"""Build recipe for the native parts of bd-cudatag_gb300.

Everything is compiled in-tree (no pip install) with plain nvcc / g++:

  libbdcudatag.so  the drop-in detector library: CUDA kernels for sm_103a
                   (csrc/*.cu) plus the C ABI and C++ API (csrc/*.cpp)
  libbdscenes.so   the seeded synthetic frame renderer used by tests and bench

Kernels are built with -fmad=false: every FP32 multiply and add is rounded
on its own, in source order, which the bit-exact comparison with the CPU
oracle relies on (the oracle is built with -ffp-contract=off).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = REPO / "include"

LIB = PKG / "libbdcudatag.so"
SCENES_LIB = PKG / "libbdscenes.so"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CUDA_SOURCES = ["k_front.cu", "k_quad.cu", "k_finalize.cu", "k_persistent.cu", "engine.cu", "noalloc.cu",
                "refine.cu"]
# The persistent kernel reads buffers that other CTAs of the same launch
# wrote: its plain global loads go to L2 (no L1 line can be stale).
EXTRA_FLAGS = {"k_persistent.cu": ["-Xptxas", "-dlcm=cg"]}
CXX_SOURCES = ["capi.cpp", "server.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + proc.stdout + proc.stderr)
        raise RuntimeError(f"build step failed: {cmd[0]} ... {cmd[-1]}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.inc")) + \
        sorted(INCLUDE.glob("bdcudatag/*.h*"))


def build_scenes(force: bool = False) -> Path:
    src = CSRC / "scenes.cpp"
    if force or _stale(SCENES_LIB, [src, CSRC / "families_data.inc"]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
              str(src), "-o", str(SCENES_LIB), "-lpthread"])
    return SCENES_LIB


# The reference-arithmetic variant: the same sources built the way the
# reference is (nvcc's default multiply-add contraction, CUDA's libm for
# sin/cos/atan2/hypot).  A test builds and loads it beside the library to
# measure how far that rounding moves results; it is not shipped.
REFARITH_LIB = PKG / "libbdcudatag_refarith.so"
REFARITH_FLAGS = ["-fmad=true", "-DBDGB_CUDA_LIBM"]


def build_library(force: bool = False, verbose_ptxas: bool = False, variant: str | None = None) -> Path:
    """Builds libbdcudatag.so, or with variant="refarith" the
    reference-arithmetic variant (own object folder and library file)."""
    if variant not in (None, "refarith"):
        raise ValueError(f"unknown build variant {variant!r}")
    build_dir = BUILD if variant is None else PKG / f"_build_{variant}"
    lib_path = LIB if variant is None else REFARITH_LIB
    fmad = ["-fmad=false"] if variant is None else REFARITH_FLAGS
    build_dir.mkdir(exist_ok=True)
    nv = nvcc()
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              "-DBDCUDATAG_BUILDING", f"-I{INCLUDE}", f"-I{CSRC}"]
    jobs = []
    objects = []
    headers = _headers()
    for name in CUDA_SOURCES:
        src = CSRC / name
        obj = build_dir / (name + ".o")
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nv, ARCH, "-lineinfo"] + fmad + ["-c", str(src), "-o", str(obj)] + common + \
                EXTRA_FLAGS.get(name, [])
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for name in CXX_SOURCES:
        src = CSRC / name
        obj = build_dir / (name + ".o")
        objects.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden",
                         "-ffp-contract=off", "-Wall", "-Wextra", "-DBDCUDATAG_BUILDING",
                         f"-I{INCLUDE}", f"-I{CSRC}", "-I/usr/local/cuda/include",
                         "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(1, len(jobs))) as pool:
        for f in [pool.submit(_run, j) for j in jobs]:
            f.result()
    if force or jobs or _stale(lib_path, objects):
        _run([nv, ARCH, "-shared", "-o", str(lib_path)] + [str(o) for o in objects] +
             ["-lcudart", "-lpthread"])
    return lib_path


def build_all(force: bool = False) -> None:
    build_scenes(force)
    build_library(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB, SCENES_LIB)
