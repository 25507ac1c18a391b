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
g++ -O2 -std=c++20 -I"$REF/detector/src" -I"$REF/detector/tests" \
    "$REF/detector/bench/scene_gen.cpp" -o "$HERE/_ref/bdcudatag_scenes"
echo "built $HERE/_ref/bdcudatag_scenes"
