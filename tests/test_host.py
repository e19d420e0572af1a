"""Host-side checks that need no GPU: the C-ABI library builds for sm_103a,
loads, and exports exactly the entry points include/forge2d_gb300.h declares;
the scene generator is deterministic; the oracle is deterministic."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from forge2d_gb300 import native, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_header_symbol(gpu_lib):
    declared = native.header_symbols()
    assert len(declared) >= 60
    assert sorted(declared) == sorted(native.SYMBOLS), "ctypes table and header disagree"
    lib = ctypes.CDLL(native.LIB_PATH)
    missing = [s for s in declared if not hasattr(lib, s)]
    assert missing == []


def test_library_exports_nothing_else(gpu_lib):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True)
    if out.returncode != 0:
        import pytest
        pytest.skip("nm unavailable")
    names = [ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()]
    ours = [n for n in names if n.startswith("f2d_")]
    assert sorted(ours) == sorted(native.header_symbols())


class Recorder:
    """A builder that records every creation call of a scene generator."""

    def __init__(self):
        self.calls = []
        self.n = 0

    def _rec(self, *a):
        self.calls.append(a)
        self.n += 1
        return self.n - 1

    def create_body(self, d):
        return self._rec("body", tuple(sorted(d.items())))

    def create_circle(self, *a):
        return self._rec("circle", repr(a))

    def create_capsule(self, *a):
        return self._rec("capsule", repr(a))

    def create_segment(self, *a):
        return self._rec("segment", repr(a))

    def create_box(self, *a):
        return self._rec("box", repr(a))

    def create_polygon(self, *a):
        return self._rec("polygon", repr(a))

    def create_revolute(self, d):
        return self._rec("revolute", tuple(sorted(d.items())))


def test_scenes_are_deterministic():
    for name, kw in (("pile", dict(count=2000, seed=1234)), ("pyramid", dict()),
                     ("pyramids_chains", dict(pyramids=2, rows=10, chains=3, links=5))):
        a, b = Recorder(), Recorder()
        scenes.build(a, name, **kw)
        scenes.build(b, name, **kw)
        assert a.calls == b.calls, name


def test_pile_mix_and_counts():
    r = Recorder()
    scenes.pile(r, count=5000, seed=1234)
    kinds = [c[0] for c in r.calls]
    assert kinds.count("body") == 5001
    n = 5000
    assert abs(kinds.count("circle") / n - 0.4) < 0.03
    assert abs(kinds.count("capsule") / n - 0.3) < 0.03
    assert abs(kinds.count("polygon") / n - 0.3) < 0.03


def test_pyramids_chains_counts():
    r = Recorder()
    scenes.pyramids_chains(r, pyramids=64, rows=40, chains=200, links=50)
    kinds = [c[0] for c in r.calls]
    assert kinds.count("revolute") == 10_000
    assert kinds.count("box") == 64 * 820 + 1
    assert kinds.count("capsule") == 10_000


def test_port_is_deterministic(port_lib):
    out = []
    for _ in range(2):
        w = port_lib.PortWorld(scenes.world_def(enableSleep=0))
        scenes.build(w, "pile", count=300, seed=5, width=20.0, height=30.0)
        for _ in range(40):
            w.step(1.0 / 60.0, 4)
        out.append(w.bodies().copy())
        w.close()
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32))
