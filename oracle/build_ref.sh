#!/usr/bin/env bash
# Builds the reference's CPU-only benchmark scene exporter from its own
# sources (detector/bench/scene_gen.cpp with the header-only scenes.hpp,
# test_support.hpp and tag_families.hpp) into oracle/_ref/.  Nothing is
# copied out of the reference tree; only the binary is written, and only in a
# container that has the reference checkout.  tests/golden/make_ref_scene_fixtures.py
# runs it to pin this project's scene renderer and the oracle.
set -euo pipefail
REF=${BD_REFERENCE_DIR:-/root/reference}
HERE=$(cd "$(dirname "$0")" && pwd)
if [ ! -d "$REF/detector/bench" ]; then
    echo "reference checkout not found at $REF; nothing to build" >&2
    exit 0
fi
mkdir -p "$HERE/_ref"
# Where the checkout was found, for the tests that read the reference's
# Python tools (tests/test_reference_consumers.py).
(cd "$REF" && pwd) > "$HERE/_ref/REFERENCE_DIR"
g++ -O2 -std=c++20 -I"$REF/detector/src" -I"$REF/detector/tests" \
    "$REF/detector/bench/scene_gen.cpp" -o "$HERE/_ref/bdcudatag_scenes"
echo "built $HERE/_ref/bdcudatag_scenes"

# The reference's own C++ consumers -- its known-answer test program and its
# benchmark -- compiled unchanged from where they lie, against this project's
# public headers and linked to this project's libbdcudatag.so.  The binaries
# are x86 and need a GPU, so they serve as a link-level drop-in check here.
LIB_DIR="$HERE/../bd-cudatag_gb300"
if [ -f "$LIB_DIR/libbdcudatag.so" ]; then
    CUDA_INC=/usr/local/cuda/include
    CUDA_LIB=/usr/local/cuda/lib64
    for prog in tests/test_detector.cpp bench/bench_detector.cpp; do
        out="$HERE/_ref/$(basename "${prog%.cpp}")_on_gb300"
        g++ -O2 -std=c++20 -I"$HERE/../include" -I"$REF/detector/src" -I"$REF/detector/tests" \
            -I"$CUDA_INC" "$REF/detector/$prog" -o "$out" \
            -L"$LIB_DIR" -lbdcudatag -L"$CUDA_LIB" -lcudart -lpthread -Wl,-rpath,"$LIB_DIR"
        echo "built $out"
    done
fi
