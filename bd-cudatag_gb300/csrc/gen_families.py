"""Generates families_data.inc: the tag36h11 and tag16h5 codeword tables.

The codewords are data defined by the AprilTag project (BSD 2-Clause, see
third_party/APRILTAG_LICENSE.md).  The detector needs them bit for bit, in the
same cell order the reference decoder uses: row-major over the data cells,
most significant bit = top-left data cell (reference
detector/src/tag_families.hpp:1-8).  This script reads that header in the
reference checkout and re-emits the numbers in this project's own table
format; it is run once, by hand, and its output is committed.

    python bd-cudatag_gb300/csrc/gen_families.py <reference checkout>/detector/src/tag_families.hpp
"""
import re
import sys
from pathlib import Path


def parse(text: str, name: str) -> list[int]:
    m = re.search(r"k%sCodes\[(\d+)\]\s*=\s*\{(.*?)\};" % name, text, re.S)
    if not m:
        raise SystemExit(f"table {name} not found")
    count = int(m.group(1))
    values = [int(v, 16) for v in re.findall(r"0x([0-9a-fA-F]+)", m.group(2))]
    if len(values) != count:
        raise SystemExit(f"{name}: expected {count} codes, parsed {len(values)}")
    return values


def emit(name: str, bits: int, values: list[int]) -> str:
    """A macro holding the initializer list, so host and __device__ arrays
    can both be defined from it."""
    width = (bits * bits + 3) // 4
    lines = [f"// {len(values)} codewords, {bits}x{bits} data cells, row-major, MSB = top-left cell",
             f"#define {name}_COUNT {len(values)}",
             f"#define {name} \\"]
    per_line = 6 if bits == 6 else 8
    for i in range(0, len(values), per_line):
        chunk = values[i:i + per_line]
        lines.append("    " + " ".join(f"0x{v:0{width}x}ull," for v in chunk) + " \\")
    lines[-1] = lines[-1][:-2]
    return "\n".join(lines)


def main() -> None:
    src = Path(sys.argv[1]).read_text()
    t36 = parse(src, "Tag36h11")
    t16 = parse(src, "Tag16h5")
    out = Path(__file__).with_name("families_data.inc")
    out.write_text(
        "// Generated by gen_families.py; do not edit.\n"
        "// Tag family codewords: data of the AprilTag project,\n"
        "// Copyright (C) 2013-2016, The Regents of The University of Michigan,\n"
        "// BSD 2-Clause license (third_party/APRILTAG_LICENSE.md).\n"
        "#pragma once\n\n"
        + emit("BD_CODEWORDS_36H11", 6, t36) + "\n\n" + emit("BD_CODEWORDS_16H5", 4, t16) + "\n")
    print(f"wrote {out} ({len(t36)} + {len(t16)} codes)")


if __name__ == "__main__":
    main()
