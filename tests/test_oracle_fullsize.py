"""The CPU restatement against the reference at the workloads' own sizes.

tests/golden/*_digests_ref.json hold, for every frame, a digest of all body
rows and colour counts of the reference stepping the 100k-body mixed pile
(first 60 frames) and the 64 pyramids plus 200 fifty-link chains (first 64
frames), recorded by tests/golden/make_golden.py. The port, stepping on its
own (no contact ids handed over), must reproduce every frame's digest.
"""
from __future__ import annotations

import json
import os

import pytest

from forge2d_gb300 import scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
DIGEST_CASES = ("pile100k", "stack_chains")


def load_digests(name):
    with open(os.path.join(GOLD, name + "_digests_ref.json")) as f:
        return json.load(f)


def frame_digest(world):
    import hashlib

    import numpy as np

    h = hashlib.sha256()
    h.update(np.ascontiguousarray(world.bodies()[:, :9], np.float32).tobytes())
    h.update(np.ascontiguousarray(world.color_counts(), np.int32).tobytes())
    return h.hexdigest()[:32]


def step_and_compare(world, gold):
    for f, want in enumerate(gold["digests"], start=1):
        world.step(1.0 / 60.0, 4)
        got = frame_digest(world)
        assert got == want, "frame %d: digest %s, reference %s" % (f, got, want)


@pytest.mark.parametrize("name", DIGEST_CASES)
def test_port_full_size_digests(port_lib, name):
    gold = load_digests(name)
    w = port_lib.PortWorld(scenes.world_def(**gold["world"]))
    scenes.build(w, gold["scene"], **gold["kw"])
    step_and_compare(w, gold)
    assert gold["contacts"][-1] > 10000
    w.close()
