"""Builds tests/golden/ref_scenes.json from the reference's own scene exporter.

Run in a container that has the reference checkout (it is not needed on the
GPU host; the JSON it writes is committed):

    oracle/build_ref.sh                      # builds oracle/_ref/bdcudatag_scenes
    python tests/golden/make_ref_scene_fixtures.py

The exporter (reference detector/bench/scene_gen.cpp) writes 32 PGM frames
and a ground-truth manifest per resolution.  The fixture keeps, per frame,
the SHA-256 of the pixels and the ground-truth ids and corners, so the tests
can check that bd-cudatag_gb300's scene renderer reproduces the reference
frames byte for byte and that the oracle and the CUDA pipeline reach the
reference's published accuracy on them (reference README.md:140-155).
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
EXPORTER = REPO / "oracle" / "_ref" / "bdcudatag_scenes"
SCENES = 32


def read_pgm(path: Path) -> tuple[int, int, bytes]:
    data = path.read_bytes()
    parts = data.split(b"\n", 3)
    assert parts[0] == b"P5"
    w, h = map(int, parts[1].split())
    assert parts[2] == b"255"
    return w, h, parts[3]


def main() -> None:
    if not EXPORTER.exists():
        subprocess.run([str(REPO / "oracle" / "build_ref.sh")], check=True)
    out: dict = {"source": "reference detector/bench/scene_gen.cpp (make_scenes, seed 6324)",
                 "scene_count": SCENES, "resolutions": {}}
    with tempfile.TemporaryDirectory() as tmp:
        subprocess.run([str(EXPORTER), tmp, str(SCENES)], check=True, capture_output=True)
        for manifest in sorted(Path(tmp).glob("scenes_*.json")):
            meta = json.loads(manifest.read_text())
            frames = []
            for scene in meta["scenes"]:
                w, h, pixels = read_pgm(Path(tmp) / scene["file"])
                assert (w, h) == (scene["width"], scene["height"])
                frames.append({"sha256": hashlib.sha256(pixels).hexdigest(),
                               "tags": [{"id": t["id"], "corners": t["corners"]}
                                        for t in scene["tags"]]})
            key = manifest.stem.replace("scenes_", "")
            out["resolutions"][key] = frames
    (HERE / "ref_scenes.json").write_text(json.dumps(out, indent=1) + "\n")
    print("wrote", HERE / "ref_scenes.json")


if __name__ == "__main__":
    main()
