#!/usr/bin/env python3
"""Write csrc/sph_mc_table.inc: the marching-cubes case table the reference's
surface extraction uses, in this library's packed form.

The reference triangulates each of the 256 corner cases with a published
case table (rtpslib/system/common/cl_src/traversehp.cl:74, `triTable`: up to
five triangles per case as edge numbers, -1 terminated).  Which diagonal
splits a quad or a pentagon is a choice the table makes, and the triangle list
the reference emits depends on it, so the library carries the same
triangulation.  This script reads it from a reference tree and packs each
case into one 64-bit word: bits 60..62 hold the triangle count, and edge e of
the case (e = 0 .. 3*count-1) sits in bits 4e..4e+3.  The generated file is
committed; run this only to regenerate it:

    python enjaparticles_gb300/mc_table_gen.py --reference <reference tree>
"""
import argparse
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "csrc", "sph_mc_table.inc")
TABLE = os.path.join("rtpslib", "system", "common", "cl_src", "traversehp.cl")


def read_table(reference):
    text = open(os.path.join(reference, TABLE), errors="replace").read()
    body = text[text.index("triTable[4096]"):]
    body = body[body.index("{") + 1:body.index("}")]
    vals = [int(v) for v in re.findall(r"-?\d+", body)]
    if len(vals) != 4096:
        raise ValueError("expected 4096 entries, found %d" % len(vals))
    return [vals[16 * c:16 * c + 16] for c in range(256)]


def pack(row):
    edges = []
    for v in row:
        if v < 0:
            break
        if not 0 <= v < 12:
            raise ValueError("edge out of range: %d" % v)
        edges.append(v)
    if len(edges) % 3 or len(edges) > 15:
        raise ValueError("bad case row %r" % (row,))
    word = (len(edges) // 3) << 60
    for e, v in enumerate(edges):
        word |= v << (4 * e)
    return word


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("RTPS_REFERENCE_TREE"))
    ap.add_argument("--out", default=OUT)
    a = ap.parse_args()
    if not a.reference:
        ap.error("give --reference or set RTPS_REFERENCE_TREE")
    words = [pack(r) for r in read_table(a.reference)]
    lines = ["// Generated by enjaparticles_gb300/mc_table_gen.py; do not edit.",
             "// The marching-cubes case table of the reference's surface extraction",
             "// (rtpslib/system/common/cl_src/traversehp.cl:74), packed one case per word:",
             "// bits 60..62 = triangle count, bits 4e..4e+3 = edge e of the case.",
             "static const unsigned long long kMcCasePacked[256] = {"]
    for c in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xull" % w for w in words[c:c + 4]) + ",")
    lines.append("};")
    with open(a.out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print(a.out)
    return 0


if __name__ == "__main__":
    sys.exit(main())
