"""The CPU restatement (oracle/port) against the committed reference fixtures.

The fixtures in tests/golden/ were recorded from the unmodified Box2D v3.1.1
sources that forge2d vendors (tests/golden/make_golden.py). Stepping the
port on its own (it keeps the reference's broadphase trees, so it creates
contacts in the reference's order) must reproduce every body state, colour
occupancy, manifold and the 256-frame penetration / kinetic-energy series
bit for bit; so must replaying the reference's contact ids through parity
mode. Runs without the reference checkout.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

from forge2d_gb300 import scenes
from parity import install_callbacks

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

CASES = {
    "pyramid": (dict(enableSleep=0), "pyramid", dict()),
    "pile": (dict(enableSleep=0, enableContinuous=1), "pile", dict(count=300, seed=11, width=30.0, height=40.0)),
    "chains": (dict(enableSleep=0), "pyramids_chains", dict(pyramids=2, rows=10, chains=6, links=20)),
    "joints": (dict(enableSleep=0), "joint_gallery", dict()),
    "joint_zoo": (dict(enableSleep=0), "joint_zoo", dict()),
    "joint_rigs": (dict(enableSleep=0), "joint_rigs", dict()),
    "joint_rigs_sleep": (dict(enableSleep=1), "joint_rigs", dict()),
    "chain_terrain": (dict(enableSleep=0, enableContinuous=0), "chain_terrain", dict(count=300)),
    "sensor_field": (dict(enableSleep=1, enableContinuous=1), "sensor_field", dict()),
    "pile_callbacks": (dict(enableSleep=1, enableContinuous=1), "pile",
                       dict(count=400, seed=6, width=20.0, height=40.0, presolve=True)),
    "pyramid_sleep": (dict(enableSleep=1), "pyramid", dict(rows=12)),
    "pile_sleep": (dict(enableSleep=1, enableContinuous=1), "pile", dict(count=300, seed=3, width=20.0, height=30.0)),
}
STATS_CASES = ("pyramid", "pile")


def frame_stats(world, mass):
    """Max penetration (-min touching separation) and total kinetic energy,
    computed exactly as tests/golden/make_golden.py does."""
    b = world.bodies()
    m = mass[:, 0].astype(np.float64)
    inertia = mass[:, 1].astype(np.float64)
    v = b[:, 4:6].astype(np.float64)
    w = b[:, 6].astype(np.float64)
    ke = float(np.sum(0.5 * m * (v * v).sum(1) + 0.5 * inertia * w * w))
    ints, fl = world.contacts()
    pen = 0.0
    if len(ints):
        sep = [fl[ints[:, 4] > k, 3 + 11 * k + 6] for k in range(2)]
        s = np.concatenate(sep)
        if len(s):
            pen = float(max(0.0, -s.min()))
    return pen, ke


def replay(world, name, frames=None, on_frame=None, plan=True):
    """Steps ``world`` through the fixture's frames (with the callback
    cases' user callbacks installed); with ``plan`` the reference's contact
    ids are handed over before each step (parity mode)."""
    gold = np.load(os.path.join(GOLD, name + "_ref.npz"))
    if name in CALLBACK_CASES:
        install_callbacks(world)
    last = int(gold["checkpoints"].max()) if frames is None else frames
    by_frame = {}
    for row in gold["plan"]:
        by_frame.setdefault(int(row[0]), []).append(row[1:])
    for f in range(1, last + 1):
        rows = by_frame.get(f)
        if rows and plan:
            world.set_contact_plan(np.array(rows, np.int32))
        world.step(1.0 / 60.0, 4)
        if on_frame is not None:
            on_frame(f)
    return gold


SENSOR_CASES = ("sensor_field",)
CALLBACK_CASES = ("pile_callbacks",)


def sensor_rows(world, f, rows):
    """Appends this step's sensor events as (frame, sensor, visitor) rows."""
    for out, ev in zip(rows, world.sensor_events()):
        out.extend((f, int(r[0]), int(r[1])) for r in ev)


def check_sensor_rows(rows, gold):
    for out, key in zip(rows, ("sensor_begin", "sensor_end")):
        got = np.array(out, np.int32).reshape(-1, 3)
        assert np.array_equal(got, gold[key]), key


def check_sets(full_rows, gold, f):
    """Solver set of every body (static, awake, sleeping set id) and its
    sleep time, where the fixture holds them."""
    if "sets_%d" % f not in gold.files:
        return
    assert np.array_equal(full_rows[:, 10], gold["sets_%d" % f]), "frame %d solver sets" % f
    assert np.array_equal(full_rows[:, 11].view(np.uint32), gold["sleep_%d" % f].view(np.uint32)), \
        "frame %d sleep times" % f


def make_port(port_lib, name):
    wkw, scene, kw = CASES[name]
    w = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(w, scene, **kw)
    return w


@pytest.mark.parametrize("plan", [False, True], ids=["native", "parity_mode"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_port_replays_reference_bit_exact(port_lib, name, plan):
    w = make_port(port_lib, name)
    gold = np.load(os.path.join(GOLD, name + "_ref.npz"))
    checks = set(int(c) for c in gold["checkpoints"])
    first = int(gold["checkpoints"][0])
    seen = []

    def on_frame(f):
        if f not in checks:
            return
        full = w.bodies()
        b = full[:, :9]
        ref = gold["bodies_%d" % f]
        assert b.shape == ref.shape
        bad = np.argwhere(b.view(np.uint32) != ref.view(np.uint32))
        assert len(bad) == 0, "frame %d: first differing (body, field) %s" % (f, bad[0].tolist())
        check_sets(full, gold, f)
        assert np.array_equal(w.color_counts(), gold["colors_%d" % f]), "frame %d colours" % f
        if f == first:
            ints, fl = w.contacts()
            assert np.array_equal(ints, gold["contact_ints_%d" % f])
            assert np.array_equal(fl.view(np.uint32), gold["contact_floats_%d" % f].view(np.uint32))
        seen.append(f)

    replay(w, name, on_frame=on_frame, plan=plan)
    assert sorted(seen) == sorted(checks)
    w.close()


@pytest.mark.parametrize("plan", [False, True], ids=["native", "parity_mode"])
@pytest.mark.parametrize("name", STATS_CASES)
def test_port_stats_series_matches_reference(port_lib, name, plan):
    """The spec statistics (per-frame max penetration and KE over 256
    frames): identical to the reference's series (tolerance 0; the bound the
    statistics are held to is 1%)."""
    ref = np.load(os.path.join(GOLD, name + "_stats_ref.npy"))
    w = make_port(port_lib, name)
    mass = w.mass()
    rows = []
    replay(w, name, frames=len(ref), on_frame=lambda f: rows.append(frame_stats(w, mass)), plan=plan)
    got = np.array(rows)
    assert np.array_equal(got, ref)
    w.close()


def test_port_hull_known_answers(port_lib):
    """Convex hull, polygon radius/centroid/normals and mass data of 40
    random point clouds equal the reference's create path (hull.c,
    geometry.c:b2MakePolygon, b2ComputePolygonMass)."""
    rows = json.load(open(os.path.join(GOLD, "hull_ref.json")))
    w = port_lib.PortWorld(scenes.world_def(enableSleep=0))
    for k, r in enumerate(rows):
        b = w.create_body(scenes.body_def(type=2, positionX=float(k * 3), positionY=0.0))
        s = w.create_polygon(b, scenes.shape_def(), r["points"], 0.0)
        assert s == r["shape"], k
        if s >= 0:
            got = w.polygon(s)
            assert np.array_equal(got.view(np.uint32), np.array(r["polygon"], np.float32).view(np.uint32)), k
        assert np.array_equal(w.mass()[b].view(np.uint32), np.array(r["mass"], np.float32).view(np.uint32)), k
    w.close()


def test_port_queries_match_reference(port_lib):
    """Ray cast and AABB overlap cases of forge2d's own tests
    (events_test.dart:152-167, :227-240), answers measured on the reference."""
    gold = json.load(open(os.path.join(GOLD, "api_ref.json")))
    w = port_lib.PortWorld(scenes.world_def(gravityY=0.0))
    bb = w.create_body(scenes.body_def(type=0, positionX=2.0))
    s = w.create_box(bb, scenes.shape_def(), 0.5, 0.5)
    assert s == gold["ray"]["shape"]
    hit = w.cast_ray_closest(0.0, 0.0, 10.0, 0.0)
    assert hit is not None
    assert [hit[0]] + hit[1].tolist() == pytest.approx(gold["ray"]["hit"], abs=1e-6)
    assert w.cast_ray_closest(0.0, 5.0, 10.0, 0.0) is None
    c1 = w.create_body(scenes.body_def(type=0, positionX=-5.0, positionY=5.0))
    s1 = w.create_circle(c1, scenes.shape_def(), 0.0, 0.0, 0.5)
    c2 = w.create_body(scenes.body_def(type=0, positionX=20.0, positionY=20.0))
    w.create_circle(c2, scenes.shape_def(), 0.0, 0.0, 0.5)
    assert s1 == gold["overlap"]["inside"]
    assert sorted(int(x) for x in w.overlap_aabb(-6.0, 4.0, -4.0, 6.0)) == gold["overlap"]["result"]
    w.close()


@pytest.mark.parametrize("name", SENSOR_CASES)
def test_port_sensor_events_match_fixture(port_lib, name):
    """Sensor begin and end events of every frame, in the reference's order
    (sensors in creation order, visitors by shape id)."""
    w = make_port(port_lib, name)
    rows = ([], [])
    gold = replay(w, name, on_frame=lambda f: sensor_rows(w, f, rows), plan=False)
    assert len(gold["sensor_begin"]) > 50 and len(gold["sensor_end"]) > 20
    check_sensor_rows(rows, gold)
    w.close()
