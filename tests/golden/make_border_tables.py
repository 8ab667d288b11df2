"""Extracts the border-copy tables of the reference's
src/shaders/probesCopyBorders.comp:21-220 (irradianceCopiesDst/Src for 8x8
colour tiles, depthCopiesDst/Src for 16x16 depth tiles) into
border_tables.json.

Run with the root of a checkout of the reference sources as its argument:
    python tests/golden/make_border_tables.py <reference checkout>
"""
import json
import os
import re
import sys


def parse(path):
    src = open(path).read()
    tables = {}
    for name in ("irradianceCopiesDst", "irradianceCopiesSrc", "depthCopiesDst", "depthCopiesSrc"):
        m = re.search(r"ivec2\s+%s\s*\[[^\]]*\]\s*=\s*\{(.*?)\};" % name, src, re.S)
        body = re.sub(r"//[^\n]*", "", m.group(1))
        pairs = re.findall(r"ivec2\(\s*(-?\d+)\s*,\s*(-?\d+)\s*\)", body)
        tables[name] = [[int(a), int(b)] for a, b in pairs]
    return tables


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_border_tables.py <reference checkout>")
    ref = sys.argv[1]
    t = parse(os.path.join(ref, "src", "shaders", "probesCopyBorders.comp"))
    t["source"] = "src/shaders/probesCopyBorders.comp:21-220"
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "border_tables.json")
    with open(out, "w") as f:
        json.dump(t, f, separators=(",", ":"))
    print(out, {k: len(v) for k, v in t.items() if isinstance(v, list)})
