"""The full-size workloads on the GPU.

Bit-exact against the reference's own per-frame digests at the workloads'
sizes (the 100k-body mixed pile, the 64 pyramids plus 200 chains), with no
reference contact ids handed over; bit-exact against the oracle over the
pile's whole 600 frames (the multithreaded restatement steps them in about
ten seconds); and
size-independent properties over a run: every step ends with status 0,
states stay finite, the run is deterministic, every colour 0..10 holds at
most one constraint per dynamic body, and the contact table holds one
contact per shape pair with 1-2 manifold points on every touching contact.
"""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import compare_contacts
from test_oracle_fullsize import DIGEST_CASES, load_digests, step_and_compare

pytestmark = pytest.mark.gpu

WKW = dict(enableSleep=0, enableContinuous=1)
PILE = dict(count=100_000, seed=1234)


def make_gpu():
    from forge2d_gb300.world import GpuWorld
    g = GpuWorld(scenes.world_def(**WKW))
    scenes.build(g, "pile", **PILE)
    return g


@pytest.mark.parametrize("name", DIGEST_CASES)
def test_gpu_full_size_digests_match_reference(gpu_lib, name):
    """Every frame's body rows and colour counts equal the reference's
    (digests recorded from the unmodified reference)."""
    from forge2d_gb300.world import GpuWorld
    gold = load_digests(name)
    g = GpuWorld(scenes.world_def(**gold["world"]))
    scenes.build(g, gold["scene"], **gold["kw"])
    step_and_compare(g, gold)
    assert g.sync() == 0
    g.close()


def test_pile100k_first_frames_bit_exact(gpu_lib, port_lib):
    g = make_gpu()
    p = port_lib.PortWorld(scenes.world_def(**WKW))
    scenes.build(p, "pile", **PILE)
    # the pile spawns in free fall: contacts appear from frame 1 on the floor
    # and between overlapping spawns
    for f in range(1, 4):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        gb, pb = g.bodies()[:, :9], p.bodies()[:, :9]
        bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
        assert len(bad) == 0, "frame %d: %s" % (f, bad[0].tolist())
    assert compare_contacts(g, p) == []
    assert np.array_equal(g.color_counts(), p.color_counts())
    g.close()
    p.close()


def test_pile100k_600_frames_bit_exact(gpu_lib, port_lib):
    """The whole scene: by frame 600 the pile holds ~3.5e5 contacts (more
    than one launch grid of threads), ~2.2e5 touching and ~1e3 overflow
    constraints."""
    g = make_gpu()
    p = port_lib.PortWorld(scenes.world_def(**WKW))
    scenes.build(p, "pile", **PILE)
    for f in range(1, 601):
        assert g.step(1.0 / 60.0, 4) == 0
        p.step(1.0 / 60.0, 4)
        if f % 150 == 0:
            gb, pb = g.bodies()[:, :9], p.bodies()[:, :9]
            bad = np.argwhere(gb.view(np.uint32) != pb.view(np.uint32))
            assert len(bad) == 0, "frame %d: %s" % (f, bad[0].tolist())
            assert np.array_equal(g.color_counts(), p.color_counts()), "frame %d" % f
    c = g.counters()
    assert c["contacts"] > 311_296 and c["overflow"] > 0, c
    assert compare_contacts(g, p) == []
    g.close()
    p.close()


def colour_property(g):
    ints, _ = g.contacts()
    _, sh = g.shapes()
    mass = g.mass()
    body_of = sh[:, 1]
    dyn = mass[:, 2] > 0.0              # inverse mass > 0: dynamic body
    col = ints[:, 3]
    touching = col >= 0
    for c in range(11):
        sel = ints[touching & (col == c)]
        if len(sel) == 0:
            continue
        ba, bb = body_of[sel[:, 1]], body_of[sel[:, 2]]
        bodies = np.concatenate([ba[dyn[ba]], bb[dyn[bb]]])
        assert len(bodies) == len(np.unique(bodies)), "colour %d reuses a dynamic body" % c
    return int(touching.sum())


def pair_property(g):
    """One contact per shape pair; touching contacts carry 1 or 2 points
    and a colour, non-touching ones none."""
    ints, _ = g.contacts()
    pairs = np.sort(ints[:, 1:3], axis=1)
    assert len(np.unique(pairs, axis=0)) == len(pairs)
    touching = (ints[:, 5] & 1) == 1
    assert ((ints[touching, 4] >= 1) & (ints[touching, 4] <= 2)).all()
    assert (ints[touching, 3] >= 0).all() and (ints[~touching, 3] == -1).all()


def test_pile100k_long_run_properties_and_determinism(gpu_lib):
    runs = []
    for rep in range(2):
        g = make_gpu()
        status = 0
        for f in range(1, 181):
            status |= g.step(1.0 / 60.0, 4)
            if rep == 0 and f in (60, 180):
                # the pile is still mostly in free fall at these frames; the
                # floor layer alone holds tens of thousands of contacts
                assert colour_property(g) > 10_000
                pair_property(g)
        status |= g.sync()
        assert status == 0
        b = g.bodies()
        assert np.isfinite(b[:, :9]).all()
        runs.append(b[:, :9].copy())
        g.close()
    assert np.array_equal(runs[0].view(np.uint32), runs[1].view(np.uint32))
