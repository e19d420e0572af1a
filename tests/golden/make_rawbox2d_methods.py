"""Lists the methods of forge2d's RawBox2D interface (the backend seam the C
ABI replaces) with their line numbers, into tests/golden/rawbox2d_methods.json.

Usage: python tests/golden/make_rawbox2d_methods.py   (needs the reference
checkout; reads packages/forge2d/lib/src/backend/raw_box2d.dart as text)
"""
from __future__ import annotations

import json
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = "/root/reference/packages/forge2d/lib/src/backend/raw_box2d.dart"

# a declaration line inside the interface: two-space indent, a return type
# (a record type in parentheses or braces included), the method name, "("
DECL = re.compile(r"^  (?!//)(?:\([^)]*\)|\(\{[^)]*\}\)|[\w<>?,\[\] ]+?)\s+([a-z]\w*)\(")


def main():
    lines = open(SRC).read().split("\n")
    start = next(i for i, l in enumerate(lines) if "abstract interface class RawBox2D" in l)
    end = start + 1
    while not lines[end].startswith("}"):
        end += 1
    methods = []
    for i in range(start + 1, end):
        m = DECL.match(lines[i])
        if m:
            methods.append({"method": m.group(1), "line": i + 1})
    out = {"source": "packages/forge2d/lib/src/backend/raw_box2d.dart", "interface_line": start + 1,
           "methods": methods}
    with open(os.path.join(HERE, "rawbox2d_methods.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(len(methods), "methods")


if __name__ == "__main__":
    main()
