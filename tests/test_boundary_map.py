"""The drop-in boundary covers forge2d's RawBox2D interface (CPU).

tests/golden/rawbox2d_methods.json lists the interface's methods as the
reference declares them (made by make_rawbox2d_methods.py from
raw_box2d.dart); tests/golden/rawbox2d_map.json maps each to the C call
(and property code) that serves it, or names why it is left out. Every
listed method must be mapped or excluded, every mapped call declared in the
header and exported by the library, every code defined in the header; the
oracle's copy of the codes must equal the header's.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden")
HEADER = os.path.join(ROOT, "include", "forge2d_gb300.h")


def _header():
    with open(HEADER) as f:
        return f.read()


def test_every_rawbox2d_method_is_mapped():
    methods = json.load(open(os.path.join(GOLD, "rawbox2d_methods.json")))["methods"]
    mapping = json.load(open(os.path.join(GOLD, "rawbox2d_map.json")))["map"]
    names = [m["method"] for m in methods]
    assert len(names) == len(set(names)) == 238
    assert set(names) == set(mapping)
    for m in methods:
        e = mapping[m["method"]]
        assert e["line"] == m["line"], m
        assert ("call" in e) != ("excluded" in e), m
    excluded = sorted(n for n, e in mapping.items() if "excluded" in e)
    assert len(excluded) <= 4, excluded


def test_mapped_calls_are_declared_and_exported():
    from forge2d_gb300 import native
    hdr = _header()
    declared = set(re.findall(r"F2D_API [^;(]*?\b(f2d_\w+)\s*\(", hdr))
    codes = set(re.findall(r"^#define (F2D_\w+) ", hdr, re.M))
    mapping = json.load(open(os.path.join(GOLD, "rawbox2d_map.json")))["map"]
    lib = C.CDLL(native.LIB_PATH)
    for name, e in mapping.items():
        for call in e.get("call", "").split():
            assert call in declared, (name, call)
            assert hasattr(lib, call), (name, call)
        for code in e.get("code", "").split():
            assert code in codes, (name, code)


def test_oracle_codes_equal_header_codes():
    pat = r"^#define (F2D_(?:BODY|SHAPE|JP)_[A-Z_]+) (\d+)"
    ours = dict(re.findall(pat, _header(), re.M))
    with open(os.path.join(ROOT, "oracle", "port", "f2d_defs.h")) as f:
        theirs = dict(re.findall(pat, f.read(), re.M))
    ours.pop("F2D_BODY_DUMP_STRIDE", None)
    theirs.pop("F2D_BODY_DUMP_STRIDE", None)
    assert ours == theirs
