"""Pins the CPU restatement to the live reference (needs the reference
checkout; skipped elsewhere, where the committed fixtures stand in).

The reference world and the port are stepped in lock step with nothing
passed between them: the port keeps the reference's broadphase trees, so it
creates contacts in the reference's order with the reference's ids. Bodies,
manifolds, colours, events, tree orders and query answers must agree bit for
bit. One case also drives the port in parity mode (the reference's contact
ids handed over before each step), which the GPU replays of recorded
fixtures use.
"""
from __future__ import annotations

import numpy as np
import pytest

from forge2d_gb300 import scenes

from parity import (blast, build_property_scene, compare_contacts, destroy_script, edit_motors, filter_rule,
                    install_callbacks, new_contacts, pre_solve_rule, property_reads, property_script, ray_answers,
                    point_answers, rounded_rays, rounded_scene, touching_pair, multishape_scene, MULTI_BLASTS, type_script)


def trees_equal(ref, port):
    for t in range(3):
        assert np.array_equal(ref.tree_order(t), port.tree_order(t)), t
        assert np.array_equal(ref.tree_stats(t), port.tree_stats(t)), (t, ref.tree_stats(t), port.tree_stats(t))


def lockstep(ref, port, frames, each=None, plan=False):
    prev = set()
    for f in range(1, frames + 1):
        ref.step(1.0 / 60.0, 4)
        if plan:
            ints, _ = ref.contacts()
            prev, created = new_contacts(prev, ints)
            if created:
                port.set_contact_plan(np.array(created, np.int32))
        port.step(1.0 / 60.0, 4)
        rb, pb = ref.bodies()[:, :9], port.bodies()[:, :9]
        bad = np.argwhere(rb.view(np.uint32) != pb.view(np.uint32))
        assert len(bad) == 0, "frame %d: body/field %s ref %r port %r" % (
            f, bad[0].tolist(), rb[tuple(bad[0])], pb[tuple(bad[0])])
        if each is not None:
            each(f)


SCENES = [
    ("pile_mixed_ccd", dict(enableSleep=0, enableContinuous=1), "pile",
     dict(count=500, seed=3, width=24.0, height=60.0), 150),
    ("pile_no_ccd", dict(enableSleep=0, enableContinuous=0), "pile",
     dict(count=400, seed=7, width=20.0, height=30.0), 120),
    ("pyramid_small", dict(enableSleep=0), "pyramid", dict(rows=12), 200),
    ("chains", dict(enableSleep=0), "pyramids_chains", dict(pyramids=3, rows=8, chains=10, links=25), 300),
    ("joint_gallery", dict(enableSleep=0), "joint_gallery", dict(copies=6), 400),
    ("joint_zoo", dict(enableSleep=0), "joint_zoo", dict(copies=4), 400),
    ("joint_rigs", dict(enableSleep=0), "joint_rigs", dict(copies=4), 400),
    # chain shapes: one-sided segments with ghost vertices, continuous
    # collision on and off (a fast body meeting several segments at once
    # visits them in the static tree's order)
    ("chain_terrain", dict(enableSleep=0, enableContinuous=0), "chain_terrain", dict(), 300),
    ("chain_terrain_ccd", dict(enableSleep=0, enableContinuous=1), "chain_terrain", dict(), 300),
]


@pytest.mark.parametrize("name,wkw,scene,kw,frames", SCENES, ids=[s[0] for s in SCENES])
def test_port_lockstep_with_reference(ref_lib, port_lib, name, wkw, scene, kw, frames):
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, scene, **kw)
    scenes.build(port, scene, **kw)

    def each(f):
        if f % 25 == 0 or f == frames:
            assert compare_contacts(ref, port) == []
            assert np.array_equal(ref.color_counts(), port.color_counts())
            trees_equal(ref, port)

    lockstep(ref, port, frames, each)
    ref.close()
    port.close()


def test_port_parity_mode_with_reference(ref_lib, port_lib):
    """Parity mode: the reference's new contact ids handed to the port before
    each step give the same world as the port's own order."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, "pile", count=300, seed=5, width=20.0, height=40.0)
    scenes.build(port, "pile", count=300, seed=5, width=20.0, height=40.0)

    def each(f):
        if f % 30 == 0:
            assert compare_contacts(ref, port) == []

    lockstep(ref, port, 120, each, plan=True)
    ref.close()
    port.close()


SLEEP_SCENES = [
    ("pyramid_sleep", dict(enableSleep=1), "pyramid", dict(rows=12), 300),
    ("pile_sleep", dict(enableSleep=1, enableContinuous=1), "pile",
     dict(count=300, seed=3, width=20.0, height=30.0), 450),
    ("chains_sleep", dict(enableSleep=1), "pyramids_chains", dict(pyramids=2, rows=6, chains=4, links=10), 400),
    ("joint_zoo_sleep", dict(enableSleep=1), "joint_zoo", dict(copies=3), 400),
    ("joint_rigs_sleep", dict(enableSleep=1), "joint_rigs", dict(copies=3), 400),
    ("chain_terrain_sleep", dict(enableSleep=1, enableContinuous=0), "chain_terrain", dict(count=200), 500),
    ("chain_terrain_ccd_sleep", dict(enableSleep=1, enableContinuous=1), "chain_terrain", dict(count=200), 500),
]


def lockstep_full(ref, port, frames, start=1):
    """Lock step comparing every body row: transform, velocity, centre,
    solver set (awake, sleeping set id) and sleep time."""
    for f in range(start, start + frames):
        ref.step(1.0 / 60.0, 4)
        port.step(1.0 / 60.0, 4)
        rb, pb = ref.bodies(), port.bodies()
        bad = np.argwhere(rb.view(np.uint32) != pb.view(np.uint32))
        assert len(bad) == 0, "frame %d: body/field %s ref %r port %r" % (
            f, bad[0].tolist(), rb[tuple(bad[0])], pb[tuple(bad[0])])
        assert ref.awake_body_count() == port.awake_body_count(), f
        if f % 25 == 0:
            assert compare_contacts(ref, port) == [], f
            assert np.array_equal(ref.color_counts(), port.color_counts()), f
            trees_equal(ref, port)


@pytest.mark.parametrize("name,wkw,scene,kw,frames", SLEEP_SCENES, ids=[s[0] for s in SLEEP_SCENES])
def test_port_sleep_lockstep_with_reference(ref_lib, port_lib, name, wkw, scene, kw, frames):
    """Islands, sleeping solver sets and the split of the sleepiest island:
    bodies fall asleep on the same frame with the same set ids."""
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, scene, **kw)
    scenes.build(port, scene, **kw)
    lockstep_full(ref, port, frames)
    if name in ("pyramid_sleep", "pile_sleep"):
        assert ref.awake_body_count() == 0
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_sensor_events_with_reference(ref_lib, port_lib, sleep):
    """b2OverlapSensors: every frame's sensor begin and end events, in order
    (static zones, a masked zone, a zone with events off, a kinematic sweeper,
    a sensor riding a falling body; visitors with and without events)."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, "sensor_field")
    scenes.build(port, "sensor_field")
    totals = [0, 0]
    for f in range(1, 301):
        lockstep_full(ref, port, 1, start=f)
        for k, (a, b) in enumerate(zip(ref.sensor_events(), port.sensor_events())):
            assert np.array_equal(a, b), (f, k)
            totals[k] += len(a)
    assert totals[0] > 100 and totals[1] > 50, totals
    ref.close()
    port.close()


def test_port_callbacks_with_reference(ref_lib, port_lib):
    """Custom filter (new pairs and continuous candidates) and pre-solve
    (one-way contacts) callbacks: bit-identical bodies, sets and contacts,
    and both callbacks reject something."""
    wkw = dict(enableSleep=1, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    seen = {"filter": 0, "pre": 0}

    def counting_filter(a, b):
        ok = filter_rule(a, b)
        seen["filter"] += not ok
        return ok

    def counting_pre(a, b, m):
        ok = pre_solve_rule(a, b, m)
        seen["pre"] += not ok
        return ok

    for w in (ref, port):
        scenes.build(w, "pile", count=400, seed=6, width=20.0, height=40.0, presolve=True)
    ref.set_custom_filter(counting_filter)
    ref.set_pre_solve(counting_pre)
    install_callbacks(port)
    lockstep_full(ref, port, 300)
    assert seen["filter"] > 100 and seen["pre"] > 100, seen
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_explode_with_reference(ref_lib, port_lib, sleep):
    """b2World_Explode three times into a settling pile (falloff, no falloff,
    a category mask), in lock step."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        scenes.build(w, "pile", count=300, seed=3, width=20.0, height=30.0)
    for f in range(1, 401):
        blast(ref, f)
        blast(port, f)
        lockstep_full(ref, port, 1, start=f)
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_motor_edits_with_reference(ref_lib, port_lib, sleep):
    """Motor speed, maximum and on/off of prismatic and wheel joints changed
    between steps (b2*Joint_EnableMotor / SetMotorSpeed / SetMax*)."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    mr, mp = [], []
    scenes.build(ref, "joint_rigs", copies=3, motors=mr)
    scenes.build(port, "joint_rigs", copies=3, motors=mp)
    assert mr == mp and len(mr) == 9
    for f in range(1, 341):
        edit_motors(ref, mr, f)
        edit_motors(port, mp, f)
        lockstep_full(ref, port, 1, start=f)
    ref.close()
    port.close()


@pytest.mark.parametrize("scene,kw", [("joint_gallery", dict(copies=2)), ("joint_zoo", dict(copies=2)),
                                      ("joint_rigs", dict(copies=2))], ids=["revolute", "weld_distance", "rigs"])
def test_port_joint_constraint_with_reference(ref_lib, port_lib, scene, kw):
    """b2Joint_GetConstraintForce / Torque of every joint, every 20 frames."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, scene, **kw)
    scenes.build(port, scene, **kw)
    nonzero = 0
    for f in range(1, 201):
        lockstep_full(ref, port, 1, start=f)
        if f % 20 == 0:
            for j in range(60):
                a, b = ref.joint_constraint(j), port.joint_constraint(j)
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (f, j, a, b)
                nonzero += bool(np.any(a != 0))
    assert nonzero > 50
    ref.close()
    port.close()


def test_port_cast_ray_callback_with_reference(ref_lib, port_lib):
    """b2World_CastRay's callback form: the closest-hit and all-hits
    callbacks end with the reference's answers."""
    wkw = dict(enableSleep=0, enableContinuous=0)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        scenes.build(w, "chain_terrain", count=150)
    lockstep_full(ref, port, 60)
    rng = np.random.default_rng(1)
    rays = [(rng.uniform(-20, 20, 2) + [0.0, 15.0], rng.uniform(-30, 30, 2)) for _ in range(150)]
    a, b = ray_answers(ref, rays), ray_answers(port, rays)
    assert a == b
    assert sum(len(x[1]) for x in a) > 100
    ref.close()
    port.close()


CHAIN_RAYS = [
    # (origin, translation): down onto the floor, up through the floor's back
    # (one-sided: no hit on it), across the ramp from both sides
    ((0.3, 30.0), (0.0, -40.0)), ((5.0, -3.0), (0.0, 60.0)), ((-21.0, 12.0), (42.0, 0.5)),
    ((12.0, 30.0), (0.0, -25.0)), ((12.0, 10.0), (0.0, 10.0)), ((-30.0, 5.0), (60.0, 0.0)),
]


def test_port_chain_queries_with_reference(ref_lib, port_lib):
    """Chain segment ids and one-sided ray casts (b2RayCastSegment with
    oneSided) agree with the reference after the pile has settled a little."""
    wkw = dict(enableSleep=0, enableContinuous=0)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    scenes.build(ref, "chain_terrain", count=100)
    scenes.build(port, "chain_terrain", count=100)
    for c in (0, 1):
        assert np.array_equal(ref.chain_segments(c), port.chain_segments(c))
    assert len(ref.chain_segments(0)) == 51 and len(ref.chain_segments(1)) == 6
    lockstep_full(ref, port, 60)
    for o, t in CHAIN_RAYS:
        rs, rf = ref.cast_ray_closest(o[0], o[1], t[0], t[1])
        ps, pf = port.cast_ray_closest(o[0], o[1], t[0], t[1])
        assert rs == ps and np.array_equal(rf.view(np.uint32), pf.view(np.uint32)), (o, t)
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_mouse_target_moves_with_reference(ref_lib, port_lib, sleep):
    """b2MouseJoint_SetTarget between steps: the held boxes follow the new
    targets (no wake: a sleeping box stays asleep) bit for bit."""
    wkw = dict(enableSleep=sleep)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    mr = scenes.build(ref, "joint_rigs", copies=3)
    mp = scenes.build(port, "joint_rigs", copies=3)
    assert mr == mp
    lockstep_full(ref, port, 60)
    for t, (dx, dy) in enumerate([(-1.5, 4.0), (2.0, 1.5), (0.5, 6.0)]):
        for w in (ref, port):
            for k, j in enumerate(mr):
                w.mouse_set_target(j, -90.0 + 5.0 + 30.0 * k + 20.0 + dx, dy)
        lockstep_full(ref, port, 80, start=61 + 80 * t)
    ref.close()
    port.close()


def test_port_wake_by_contact_and_api(ref_lib, port_lib):
    """A sleeping pyramid woken by falling bodies created later (its set's
    contacts and joints re-enter the graph inside the serial contact update),
    then bodies put to sleep and woken through b2Body_SetAwake, then
    sleeping disabled world-wide."""
    wkw = dict(enableSleep=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        scenes.build(w, "pyramid", rows=10)
        scenes.build(w, "pyramids_chains", pyramids=1, rows=4, chains=3, links=6, gap=30.0)
    lockstep_full(ref, port, 150)
    assert ref.awake_body_count() < 30
    for w in (ref, port):
        b = w.create_body(scenes.body_def(type=scenes.DYNAMIC, positionX=0.3, positionY=14.0))
        w.create_circle(b, scenes.shape_def(), 0.0, 0.0, 0.5)
        b2 = w.create_body(scenes.body_def(type=scenes.DYNAMIC, positionX=-3.2, positionY=16.0))
        w.create_box(b2, scenes.shape_def(), 0.4, 0.4)
    lockstep_full(ref, port, 120, start=151)
    for w in (ref, port):
        w.set_awake(5, False)
        w.set_awake(30, True)
    lockstep_full(ref, port, 40, start=271)
    for w in (ref, port):
        w.enable_sleeping(False)
    assert ref.awake_body_count() == port.awake_body_count()
    lockstep_full(ref, port, 40, start=311)
    ref.close()
    port.close()


def hit_rows(w):
    ints, fl = w.hit_events()
    return sorted(tuple(i) + tuple(f) for i, f in zip(ints.tolist(), fl.view(np.uint32).tolist()))


def test_port_events_match_reference(ref_lib, port_lib):
    """Begin/end touch events, hit events and body move events per frame
    (contact.c:500-560, solver.c:1740-1800, body move events world.c)."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    kw = dict(count=200, seed=21, width=16.0, height=20.0, enable_hit_events=True, enable_contact_events=True)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        scenes.build(w, "pile", **kw)

    totals = np.zeros(4, np.int64)

    def each(f):
        assert np.array_equal(ref.event_counts(), port.event_counts()), f
        for a, b in ((ref.begin_events(), port.begin_events()), (ref.end_events(), port.end_events())):
            assert np.array_equal(a, b), f
        # begin events carry the manifold of the collide phase, bit for bit
        rm, pm = ref.begin_manifolds(), port.begin_manifolds()
        assert np.array_equal(rm.view(np.uint32), pm.view(np.uint32)), f
        # hit events: same multiset; the order inside one colour follows the
        # reference's colour arrays, which the port does not keep
        assert hit_rows(ref) == hit_rows(port), f
        ri, rf = ref.move_events()
        pi, pf = port.move_events()
        assert np.array_equal(ri, pi) and np.array_equal(rf.view(np.uint32), pf.view(np.uint32)), f
        totals[:] += ref.event_counts()

    lockstep(ref, port, 90, each)
    assert totals[0] > 0 and totals[1] > 0 and totals[2] > 0 and totals[3] > 0
    ref.close()
    port.close()


def test_port_queries_on_moving_scene(ref_lib, port_lib):
    """Closest-ray and AABB-overlap answers over a settling pile."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    kw = dict(count=300, seed=4, width=20.0, height=20.0)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        scenes.build(w, "pile", **kw)
    rng = np.random.default_rng(9)
    hits = [0]

    def each(f):
        if f % 10:
            return
        for _ in range(20):
            o = rng.uniform(-12, 12, 2)
            t = rng.uniform(-15, 15, 2)
            a = ref.cast_ray_closest(o[0], o[1], t[0], t[1])
            b = port.cast_ray_closest(o[0], o[1], t[0], t[1])
            assert (a is None) == (b is None)
            if a is not None:
                hits[0] += 1
                assert a[0] == b[0]
                assert np.array_equal(a[1].view(np.uint32), b[1].view(np.uint32))
            lo = rng.uniform(-12, 8, 2)
            hi = lo + rng.uniform(0.1, 6, 2)
            assert sorted(ref.overlap_aabb(lo[0], lo[1], hi[0], hi[1]).tolist()) == \
                sorted(port.overlap_aabb(lo[0], lo[1], hi[0], hi[1]).tolist())

    lockstep(ref, port, 60, each)
    assert hits[0] > 20
    ref.close()
    port.close()


def build_destroy_scene(w):
    """pyramids with chains, one body with two shapes, two chain shapes on a
    static body; returns the ids the destroy script picks."""
    scenes.build(w, "pyramids_chains", pyramids=2, rows=8, chains=4, links=10, gap=3.0)
    twin = w.create_body(scenes.body_def(type=2, positionX=-2.0, positionY=9.0))
    twin_box = w.create_box(twin, scenes.shape_def(enableContactEvents=1), 0.5, 0.3)
    second = w.create_circle(twin, scenes.shape_def(density=2.0), 0.6, 0.0, 0.3)
    ground = w.create_body(scenes.body_def(type=0, positionY=-6.0))
    w.create_chain(ground, [(-40.0, 0.0), (-20.0, -1.0), (0.0, 0.0), (20.0, -1.0), (40.0, 0.0)])
    w.create_chain(ground, [(-40.0, -3.0), (-20.0, -4.0), (0.0, -3.0), (20.0, -4.0), (40.0, -3.0)])
    nb = len(w.bodies())
    return {"box": 12, "link": nb // 2, "shape": second, "joint": 5, "chain": 1, "last": nb - 3,
            "twin_box": twin_box}


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_destroy_path_with_reference(ref_lib, port_lib, sleep):
    """b2DestroyBody / b2DestroyShape / b2DestroyJoint / b2DestroyChain
    between steps, ids reused by bodies created after them, and a joint
    created between touching bodies (its bodies' contacts end): bodies,
    solver sets, contacts, colours, trees and end events in lock step."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    ids = build_destroy_scene(ref)
    assert build_destroy_scene(port) == ids
    ends = 0
    for f in range(1, 141):
        if f == 90:
            ids["touch"] = touching_pair(ref)
            assert ids["touch"] == touching_pair(port) and ids["touch"] is not None
        destroy_script(ref, f, ids)
        destroy_script(port, f, ids)
        lockstep_full(ref, port, 1, start=f)
        assert np.array_equal(ref.end_events(), port.end_events()), f
        ends += len(ref.end_events())
        if f % 10 == 0:
            assert compare_contacts(ref, port) == [], f
            assert np.array_equal(ref.color_counts(), port.color_counts()), f
            trees_equal(ref, port)
    assert ends > 0
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_type_changes_with_reference(ref_lib, port_lib, sleep):
    """b2Body_SetType / b2Body_Disable / b2Body_Enable between steps (type
    script of parity.py): bodies with their solver sets, contacts, colours,
    trees and end events in lock step, with and without sleeping."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    assert build_destroy_scene(ref) == build_destroy_scene(port)
    events = 0
    for f in range(1, 141):
        type_script(ref, f)
        type_script(port, f)
        lockstep_full(ref, port, 1, start=f)
        assert np.array_equal(ref.end_events(), port.end_events()), f
        assert np.array_equal(ref.begin_events(), port.begin_events()), f
        events += len(ref.end_events()) + len(ref.begin_events())
        if f % 5 == 0:
            assert compare_contacts(ref, port) == [], f
            assert np.array_equal(ref.color_counts(), port.color_counts()), f
            trees_equal(ref, port)
    assert events > 0
    ref.close()
    port.close()


def test_port_type_change_colour_deviation(ref_lib, port_lib):
    """The one deviation of the type change: a static chain link holding two
    joints of the constraint graph turned dynamic. The reference re-colours
    its joints one by one and each graph removal clears both bodies' colour
    bits (constraint_graph.c:303-308), including the bit the previous joint
    of this (no longer static) body just took, so two joints of one dynamic
    body end in one colour. Here a removal clears only the bits its colouring
    set: the joints get different colours and the bodies agree up to that
    step only."""
    calls = {30: (5, 0), 35: (6, 0), 45: (5, 2)}
    ws = [ref_lib.RefWorld(scenes.world_def(enableSleep=0)), port_lib.PortWorld(scenes.world_def(enableSleep=0))]
    for w in ws:
        scenes.chain(w, 0.0, 5.0, links=10)
    for f in range(1, 46):
        for w in ws:
            if f in calls:
                w.body_set_type(*calls[f])
        if f < 45:
            for w in ws:
                w.step(1.0 / 60.0, 4)
            assert np.array_equal(ws[0].bodies().view(np.uint32), ws[1].bodies().view(np.uint32)), f
    ref_colors = [ws[0].joint_color(j) for j in (4, 5)]
    port_colors = [ws[1].joint_color(j) for j in (4, 5)]
    assert ref_colors[0] == ref_colors[1]       # joints 4-5 and 5-6 share body 5 and a colour
    assert port_colors[0] != port_colors[1]
    for w in ws:
        w.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_properties_with_reference(ref_lib, port_lib, sleep):
    """The generic property calls: joint setters of every type (springs,
    limits, motors, targets, lengths, offsets, stiffness; impulses cleared
    as the reference clears them), body damping / gravity scale / bullet /
    fixed rotation / mass data, shape friction / restitution / density /
    event flags / filters (proxies re-created or moved), chain friction.
    Bodies, contacts, colours, every getter and shape point tests agree bit
    for bit in lock step."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    nb, nj = build_property_scene(ref)
    assert build_property_scene(port) == (nb, nj)
    ns = len(ref.shapes()[1])
    for f in range(1, 101):
        property_script(ref, f, nb, nj)
        property_script(port, f, nb, nj)
        lockstep_full(ref, port, 1, start=f)
        assert np.array_equal(ref.end_events(), port.end_events()), f
        if f % 10 == 0:
            assert compare_contacts(ref, port) == [], f
            assert np.array_equal(ref.color_counts(), port.color_counts()), f
            a = np.array(property_reads(ref, nb, ns, nj), np.float64)
            b = np.array(property_reads(port, nb, ns, nj), np.float64)
            bad = np.flatnonzero(a.view(np.uint64) != b.view(np.uint64))
            assert len(bad) == 0, (f, bad[:5], a[bad[:5]], b[bad[:5]])
            assert point_answers(ref) == point_answers(port), f
    ref.close()
    port.close()



def test_port_rounded_polygon_rays_with_reference(ref_lib, port_lib):
    """Rays against rounded boxes and polygons take the reference's shape
    cast (conservative advancement on GJK distance): closest and all hits,
    points, normals and fractions bit for bit."""
    wkw = dict(enableSleep=0, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        rounded_scene(w)
    lockstep_full(ref, port, 40)
    rays = rounded_rays()
    a, b = ray_answers(ref, rays), ray_answers(port, rays)
    assert a == b
    assert sum(len(x[1]) for x in a) > 100
    ref.close()
    port.close()


@pytest.mark.parametrize("sleep", [0, 1])
def test_port_explode_multishape_with_reference(ref_lib, port_lib, sleep):
    """Explosions over bodies of several shapes each, through sleeping sets:
    the shapes are visited in the dynamic tree's query order, which fixes
    the order sets wake in and the order a body's impulses add up."""
    wkw = dict(enableSleep=sleep, enableContinuous=1)
    ref = ref_lib.RefWorld(scenes.world_def(**wkw))
    port = port_lib.PortWorld(scenes.world_def(**wkw))
    for w in (ref, port):
        multishape_scene(w)
    for f in range(1, 321):
        if f in MULTI_BLASTS:
            x, y, r, fo, ipl, mask = MULTI_BLASTS[f]
            for w in (ref, port):
                w.explode(x, y, r, fo, ipl, mask=mask)
        lockstep_full(ref, port, 1, start=f)
    ref.close()
    port.close()
